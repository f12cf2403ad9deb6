// C ABI entry points of libpfemgpu.so (declared in include/pfem_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <new>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"
#include "pfg_fst.cuh"

namespace pfg {

int fail(pfg_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_fail(pfg_ctx* c, cudaError_t e, const char* what) {
    return fail(c, PFG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int ensure(pfg_ctx* c, DBuf& b, size_t bytes) {
    if (bytes <= b.cap) return PFG_OK;
    size_t newcap = std::max(bytes, b.cap + b.cap / 4);
    newcap = (newcap + 255) & ~(size_t)255;
    if (c->prm.hbm_budget_bytes && c->bytes_in_use - b.cap + newcap > c->prm.hbm_budget_bytes)
        return fail(c, PFG_ERR_NOMEM, "HBM budget of %zu bytes exceeded", c->prm.hbm_budget_bytes);
    if (b.p) {
        cudaStreamSynchronize(c->stream);
        cudaFree(b.p);
        c->bytes_in_use -= b.cap;
        b.p = nullptr;
        b.cap = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, newcap);
    if (e != cudaSuccess) return fail(c, PFG_ERR_NOMEM, "cudaMalloc(%zu): %s", newcap, cudaGetErrorString(e));
    b.p = p;
    b.cap = newcap;
    c->bytes_in_use += newcap;
    return PFG_OK;
}

static cudaEvent_t take_event(pfg_ctx* c) {
    if (c->ev_used == c->ev_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        c->ev_pool.push_back(e);
    }
    return c->ev_pool[c->ev_used++];
}

void prof_begin(pfg_ctx* c, int phase) {
    if (!c->prof) return;
    if (c->ev_used + 2 > 4096) prof_flush(c);
    cudaEvent_t e = take_event(c);
    if (!e) return;
    cudaEventRecord(e, c->stream);
    c->marks.push_back(phase);
    c->marks.push_back((int)c->ev_used - 1);
    c->marks.push_back(-1);
}

void prof_end(pfg_ctx* c, int phase) {
    if (!c->prof || c->marks.size() < 3) return;
    // close the most recent open mark of this phase
    for (size_t i = c->marks.size(); i >= 3; i -= 3) {
        if (c->marks[i - 3] == phase && c->marks[i - 1] < 0) {
            cudaEvent_t e = take_event(c);
            if (!e) return;
            cudaEventRecord(e, c->stream);
            c->marks[i - 1] = (int)c->ev_used - 1;
            return;
        }
    }
}

int prof_flush(pfg_ctx* c) {
    if (c->marks.empty()) {
        c->ev_used = 0;
        return PFG_OK;
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i + 2 < c->marks.size(); i += 3) {
        const int ph = c->marks[i], a = c->marks[i + 1], b = c->marks[i + 2];
        if (b < 0) continue;
        float ms = 0;
        if (cudaEventElapsedTime(&ms, c->ev_pool[a], c->ev_pool[b]) == cudaSuccess) {
            c->phase_ms[ph] += ms;
            c->phase_n[ph] += 1;
        }
    }
    c->marks.clear();
    c->ev_used = 0;
    return PFG_OK;
}

void release(DBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

// Gauss rules of the element kernels (3 points in 2D, 4 in 3D; MomContEquation.inl:12-23)
// with the reference's decimal values (Mesh.cpp:375-378, :396-399, :444, :459, :480-483).
GaussConst gauss_const(int dim) {
    GaussConst g{};
    if (dim == 2) {
        g.n = 3;
        const double p[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}, {2.0 / 3.0, 1.0 / 6.0}};
        for (int k = 0; k < 3; ++k) {
            g.w[k] = 1.0 / 3.0;
            g.N[k][0] = 1 - p[k][0] - p[k][1];
            g.N[k][1] = p[k][0];
            g.N[k][2] = p[k][1];
        }
        g.refSize = 0.5;
    } else {
        g.n = 4;
        const double a = 0.585410196624968, b = 0.138196601125011;
        const double p[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
        for (int k = 0; k < 4; ++k) {
            g.w[k] = 0.25;
            g.N[k][0] = 1 - p[k][0] - p[k][1] - p[k][2];
            g.N[k][1] = p[k][0];
            g.N[k][2] = p[k][1];
            g.N[k][3] = p[k][2];
        }
        g.refSize = 0.16666666666666666666666666666667;
    }
    const int npe = dim + 1;
    g.sumw = 0;
    for (int k = 0; k < g.n; ++k) g.sumw += g.w[k];
    for (int i = 0; i < npe; ++i) {
        g.s[i] = 0;
        for (int k = 0; k < g.n; ++k) g.s[i] += g.w[k] * g.N[k][i];
        for (int j = 0; j < npe; ++j) {
            g.MM[i][j] = 0;
            for (int k = 0; k < g.n; ++k) g.MM[i][j] += g.N[k][i] * g.N[k][j] * g.w[k];
        }
    }
    return g;
}

}  // namespace pfg

using namespace pfg;

namespace {

__global__ void k_scatter_dirichlet(int n, const int* __restrict__ nodes, const double* __restrict__ vals, int N,
                                    int dim, double* __restrict__ vbc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int node = nodes[i];
    for (int d = 0; d < dim; ++d) vbc[(size_t)d * N + node] = vals[(size_t)d * n + i];
}

int check_ctx(pfg_ctx* c) {
    if (!c) return PFG_ERR_INVALID;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
    return PFG_OK;
}

// Surface tension needs the facets of the current mesh.
int check_facets(pfg_ctx* c) {
    if (fst_on(c) && !c->has_facets)
        return fail(c, PFG_ERR_STATE, "surface tension: call pfg_upload_facets after pfg_upload_mesh");
    return PFG_OK;
}

}  // namespace

extern "C" {

PFG_API const char* pfg_version(void) { return "pfem_gb300 0.1 (sm_103a)"; }

PFG_API const char* pfg_phase_name(int32_t phase) {
    static const char* names[PFG_NUM_PHASES] = {
        "WC predict", "WC continuity element", "WC continuity node", "WC momentum element", "WC momentum node",
        "WC time step", "PSPG element prep", "PSPG right-hand side", "PSPG matrix", "Krylov iteration",
        "Picard residual", "Position update", "Krylov SpMV", "Multigrid cycle", "Multigrid setup",
        "Heat assembly", "Heat CG SpMV"};
    return (phase >= 0 && phase < PFG_NUM_PHASES) ? names[phase] : "";
}

PFG_API int pfg_set_profiling(pfg_ctx* c, int32_t enable) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prof && !enable) prof_flush(c);
    c->prof = enable != 0;
    return PFG_OK;
}

PFG_API int pfg_get_phase_times(pfg_ctx* c, double* ms, int64_t* launches) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if ((rc = prof_flush(c))) return rc;
    for (int i = 0; i < PFG_NUM_PHASES; ++i) {
        if (ms) ms[i] = c->phase_ms[i];
        if (launches) launches[i] = c->phase_n[i];
    }
    return PFG_OK;
}

PFG_API int pfg_set_tuning(pfg_ctx* c, const pfg_tuning* t) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!t) return fail(c, PFG_ERR_INVALID, "null tuning");
    pfg_tuning n = c->tune;
    const int lanes0 = c->dim == 2 ? 4 : 8;
    if (t->spmv_lanes) {
        if (t->spmv_lanes != lanes0 / 2 && t->spmv_lanes != lanes0 && t->spmv_lanes != 2 * lanes0)
            return fail(c, PFG_ERR_INVALID, "spmv_lanes must be %d, %d or %d", lanes0 / 2, lanes0, 2 * lanes0);
        n.spmv_lanes = t->spmv_lanes;
    }
    if (t->mg_lanes) {
        if (t->mg_lanes != lanes0 / 2 && t->mg_lanes != lanes0 && t->mg_lanes != 2 * lanes0)
            return fail(c, PFG_ERR_INVALID, "mg_lanes must be %d, %d or %d", lanes0 / 2, lanes0, 2 * lanes0);
        n.mg_lanes = t->mg_lanes;
    }
    auto block_ok = [](int b) { return b == 64 || b == 128 || b == 256; };
    if (t->pair_block) {
        if (!block_ok(t->pair_block)) return fail(c, PFG_ERR_INVALID, "pair_block must be 64, 128 or 256");
        n.pair_block = t->pair_block;
    }
    if (t->elem_block) {
        if (!block_ok(t->elem_block)) return fail(c, PFG_ERR_INVALID, "elem_block must be 64, 128 or 256");
        n.elem_block = t->elem_block;
    }
    if (t->res_block) {
        if (t->res_block != 32 && t->res_block != 64) return fail(c, PFG_ERR_INVALID, "res_block must be 32 or 64");
        n.res_block = t->res_block;
    }
    c->tune = n;
    if (c->prm.kind == PFG_KIND_INCOMP_PSPG && c->prm.precision == PFG_PREC_MIXED && c->has_mesh)
        mx_release_graph(c);  // the captured Krylov chunks hold the previous launch shapes
    return PFG_OK;
}

PFG_API int pfg_get_tuning(pfg_ctx* c, pfg_tuning* t) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!t) return fail(c, PFG_ERR_INVALID, "null tuning");
    *t = c->tune;
    return PFG_OK;
}

PFG_API int pfg_get_spmv_pairs(pfg_ctx* c, int64_t* pairs) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!pairs) return fail(c, PFG_ERR_INVALID, "null pointer");
    if ((rc = prof_flush(c))) return rc;
    *pairs = c->spmv_pairs;
    return PFG_OK;
}

PFG_API int pfg_reset_phase_times(pfg_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if ((rc = prof_flush(c))) return rc;
    for (int i = 0; i < PFG_NUM_PHASES; ++i) {
        c->phase_ms[i] = 0;
        c->phase_n[i] = 0;
    }
    c->spmv_pairs = 0;
    return PFG_OK;
}

PFG_API int pfg_default_params(int32_t kind, int32_t dim, pfg_params* p) {
    if (!p || (dim != 2 && dim != 3) || (kind != PFG_KIND_INCOMP_PSPG && kind != PFG_KIND_WC_CDS_DPDT))
        return PFG_ERR_INVALID;
    std::memset(p, 0, sizeof(*p));
    p->dim = dim;
    p->kind = kind;
    p->precision = PFG_PREC_FP64;
    p->linear_solver = PFG_LINSOLVE_BICGSTAB;
    p->gravity[dim - 1] = -9.81;
    p->mu = 1e-3;
    p->rho = 1000.0;
    p->picard_max_iter = 10;
    p->residual = PFG_RES_AX_F;
    p->picard_min_res = 1e-6;
    p->krylov_max_iter = 5000;
    p->krylov_rel_tol = 1e-14;
    p->krylov_abs_tol = 1e-10;
    p->heat_max_iter = 10;
    p->heat_min_res = 1e-6;
    p->heat_residual = PFG_RES_T;
    p->refine_max_iter = 30;
    // measured: a 330k-node 3D dam break steps 14% faster at 1e-4, the 2D cases 11% faster at 1e-3
    p->inner_rel_tol = dim == 3 ? 5e-4 : 1e-3;
    p->preconditioner = PFG_PC_MULTIGRID;
    p->K0 = 2.2e7;
    p->K0p = 7.0;
    p->rho_star = 1000.0;
    p->security_coeff = 0.3;
    p->max_dt = 1e-3;
    p->meduri = 1;
    p->hbm_budget_bytes = 0;
    return PFG_OK;
}

PFG_API int pfg_create(const pfg_params* params, pfg_ctx** out) {
    if (!params || !out) return PFG_ERR_INVALID;
    *out = nullptr;
    if (params->dim != 2 && params->dim != 3) return PFG_ERR_INVALID;
    if (params->kind != PFG_KIND_INCOMP_PSPG && params->kind != PFG_KIND_WC_CDS_DPDT) return PFG_ERR_INVALID;
    if (params->precision != PFG_PREC_FP64 && params->precision != PFG_PREC_MIXED) return PFG_ERR_INVALID;
    if (params->linear_solver != PFG_LINSOLVE_BICGSTAB && params->linear_solver != PFG_LINSOLVE_LU)
        return PFG_ERR_INVALID;
    // the direct solver is the plain form's (the mixed form refines FP32 Krylov corrections)
    if (params->linear_solver == PFG_LINSOLVE_LU &&
        (params->kind != PFG_KIND_INCOMP_PSPG || params->precision != PFG_PREC_FP64))
        return PFG_ERR_UNSUPPORTED;
    if (params->tau0 < 0 || (params->tau0 > 0 && !(params->m_reg > 0))) return PFG_ERR_INVALID;
    if (params->tau0 > 0 && params->kind != PFG_KIND_INCOMP_PSPG) return PFG_ERR_UNSUPPORTED;  // Bingham: PSPG only
    // Boussinesq coupling: problem "Boussinesq" (PSPG) or "BoussinesqWC" (WC, plain FP64 form)
    if (params->boussinesq != 0 && params->boussinesq != 1) return PFG_ERR_INVALID;
    if (params->boussinesq && params->kind == PFG_KIND_WC_CDS_DPDT) {
        if (params->precision != PFG_PREC_FP64) return PFG_ERR_UNSUPPORTED;
        if (!(params->heat_cv > 0) || !(params->heat_k >= 0)) return PFG_ERR_INVALID;
    }
    if (params->heat_fs_flags & ~(PFG_HEAT_Q | PFG_HEAT_QH | PFG_HEAT_QR)) return PFG_ERR_INVALID;
    if (params->heat_residual != PFG_RES_T && params->heat_residual != PFG_RES_AX_F) return PFG_ERR_INVALID;
    if (params->heat_phase_change && !(params->heat_dt_melt > 0)) return PFG_ERR_INVALID;
    if (params->assembly != PFG_ASM_FP32 && params->assembly != PFG_ASM_DOUBLE_FLOAT) return PFG_ERR_INVALID;
    // fractional step: the plain FP64 form of the incompressible solver, U or U_P residual
    // (the reference throws for Ax_f, MomContEquationFracStep.inl:626-628)
    if (params->frac_step != 0 && params->frac_step != 1) return PFG_ERR_INVALID;
    if (params->frac_step) {
        if (params->kind != PFG_KIND_INCOMP_PSPG || params->precision != PFG_PREC_FP64 ||
            params->linear_solver != PFG_LINSOLVE_BICGSTAB || params->boussinesq)
            return PFG_ERR_UNSUPPORTED;
        if (!(params->gamma_fs >= 0 && params->gamma_fs <= 1)) return PFG_ERR_INVALID;
        if (params->residual != PFG_RES_U && params->residual != PFG_RES_U_P) return PFG_ERR_INVALID;
    }
    // continuity forms of the WC solver: the density forms in the plain FP64 form
    if (params->wc_version < PFG_WC_DPDT || params->wc_version > PFG_WC_DRHODT) return PFG_ERR_INVALID;
    if (params->wc_version != PFG_WC_DPDT &&
        (params->kind != PFG_KIND_WC_CDS_DPDT || params->precision != PFG_PREC_FP64))
        return PFG_ERR_UNSUPPORTED;
    pfg_ctx* c = new (std::nothrow) pfg_ctx();
    if (!c) return PFG_ERR_NOMEM;
    c->prm = *params;
    c->dim = params->dim;
    c->npe = params->dim + 1;
    // pair assembly: the row-staged kernel (128) in 3D, where a pair has ~5 element items; in 2D
    // (~2 items per pair) the pair-parallel kernel reading global memory (64) does as well or
    // better; 256 = item-parallel.  The autotuner compares the three.
    c->tune = pfg_tuning{params->dim == 2 ? 4 : 8, params->dim == 2 ? 64 : 128, BLOCK, 64, params->dim == 2 ? 4 : 8};
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_scalars, 64 * sizeof(double));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) {
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return PFG_ERR_CUDA;
    }
    c->max_grid = c->num_sms * 8;
    if (ensure(c, c->err_word, 64) || ensure(c, c->red, sizeof(double) * (size_t)(c->max_grid * 4 + 256))) {
        pfg_destroy(c);
        return PFG_ERR_NOMEM;
    }
    cudaMemsetAsync(c->red.p, 0, c->red.cap, c->stream);
    cudaMemsetAsync(c->err_word.p, 0, c->err_word.cap, c->stream);
    cudaStreamSynchronize(c->stream);
    *out = c;
    return PFG_OK;
}

PFG_API int pfg_destroy(pfg_ctx* c) {
    if (!c) return PFG_ERR_INVALID;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    DBuf* bufs[] = {&c->pos, &c->pos_save, &c->flags, &c->conn, &c->ne_ptr, &c->ne_elem, &c->ne_loc,
                    &c->nbr_ptr, &c->nbr, &c->pair_node, &c->row_ptr, &c->col, &c->val, &c->val32,
                    &c->diag_pos, &c->rhs, &c->edata, &c->edata_df, &c->q, &c->q_prev, &c->q_iter_prev,
                    &c->vbc, &c->kv, &c->kv32, &c->binv, &c->red, &c->err_word, &c->ws, &c->wc_el, &c->wc_dt,
                    &c->stage, &c->wc_eld, &c->wc_nodal, &c->inc_slot, &c->binv32, &c->node_inst,
                    &c->mx_seg, &c->mx_ii, &c->mx_id, &c->mx_sc, &c->mx_part, &c->mx_cnt, &c->mx_scale,
                    &c->mx_list, &c->fc_nodes, &c->fc_elem, &c->nf_nodes, &c->nf_ptr, &c->nf_ent, &c->fst_force,
                    &c->mg_x0, &c->mg_in64, &c->val16, &c->heat_t, &c->heat_flags, &c->heat_tbc, &c->heat_val,
                    &c->heat_rhs, &c->heat_cg, &c->heat_red, &c->heat_cg32, &c->heat_rhs32, &c->hf_ptr, &c->hf_ent, &c->hf_fflags, &c->heat_q,
                    &c->pe_ptr, &c->pe_item, &c->pe_pair, &c->pe_pos, &c->el_slot, &c->ne_slot, &c->conn_s, &c->mx_scale32, &c->mx_f32, &c->mx_xdf, &c->mx_vpdf, &c->mx_tdf,
                    &c->mx_rec, &c->mx_gdf, &c->wc_inst, &c->mx_ed_aos, &c->mx_vsum, &c->wch_rec, &c->fs_gauge, &c->fs_rp, &c->fs_col, &c->fs_val, &c->fs_lval, &c->fs_mval, &c->fs_vec, &c->fs_cg, &c->fs_red, &c->lu_front, &c->lu_nodes,
                    &c->lu_recs, &c->lu_kids, &c->lu_maps, &c->lu_piv, &c->lu_mat, &c->lu_vec, &c->lu_list,
                    &c->lu_r, &c->lu_one};
    wc_release_graphs(c);
    mg_release(c);
    mx_release_graph(c);
    for (DBuf* b : bufs) release(*b);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->h_scalars) cudaFreeHost(c->h_scalars);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PFG_OK;
}

PFG_API const char* pfg_last_error(const pfg_ctx* c) { return c ? c->err.c_str() : "null context"; }

PFG_API int pfg_upload_mesh(pfg_ctx* c, int32_t n_nodes, const double* pos, const uint8_t* flags, int32_t n_elems,
                            const int32_t* conn) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (n_nodes <= 0 || n_elems < 0 || !pos || !flags || (n_elems > 0 && !conn))
        return fail(c, PFG_ERR_INVALID, "pfg_upload_mesh: invalid sizes or null pointers");
    const int npe = c->npe, dim = c->dim;
    // validate connectivity on the host: indices in range and distinct within an element
    for (int e = 0; e < n_elems; ++e) {
        for (int k = 0; k < npe; ++k) {
            const int v = conn[(size_t)k * n_elems + e];
            if (v < 0 || v >= n_nodes) return fail(c, PFG_ERR_INVALID, "element %d references node %d", e, v);
            for (int j = 0; j < k; ++j)
                if (conn[(size_t)j * n_elems + e] == v)
                    return fail(c, PFG_ERR_INVALID, "element %d repeats node %d", e, v);
        }
    }
    c->has_mesh = false;
    c->has_system = false;
    lu_release(c);
    c->N = n_nodes;
    c->E = n_elems;
    c->R = (dim + 1) * n_nodes;
    c->nstates = (c->prm.kind == PFG_KIND_INCOMP_PSPG) ? (dim + 1) : (2 * dim + 2);
    const size_t N = n_nodes, E = n_elems;
    if ((rc = ensure(c, c->pos, sizeof(double) * dim * N)) || (rc = ensure(c, c->pos_save, sizeof(double) * dim * N)) ||
        (rc = ensure(c, c->flags, N)) || (rc = ensure(c, c->conn, sizeof(int) * std::max<size_t>(npe * E, 1))) ||
        (rc = ensure(c, c->vbc, sizeof(double) * dim * N)))
        return rc;
    c->h_flags.assign(flags, flags + N);
    c->h_conn.assign(conn, conn + (size_t)npe * E);
    c->has_facets = false;
    c->h_facets.clear();
    c->h_facet_elm.clear();
    c->F = 0;
    c->n_fst_nodes = 0;
    PFG_CUDA(c, cudaMemcpyAsync(c->pos.p, pos, sizeof(double) * dim * N, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->pos_save.p, pos, sizeof(double) * dim * N, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->flags.p, flags, N, cudaMemcpyHostToDevice, c->stream));
    if (E) PFG_CUDA(c, cudaMemcpyAsync(c->conn.p, conn, sizeof(int) * npe * E, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->vbc.p, 0, sizeof(double) * dim * N, c->stream));
    if ((rc = build_topology(c))) return rc;
    if (c->prm.kind == PFG_KIND_INCOMP_PSPG) {
        if ((rc = pspg_alloc(c)) || (rc = krylov_alloc(c))) return rc;
        if (c->prm.frac_step && (rc = fs_alloc(c))) return rc;
        // heat buffers: allocated with the mesh for Boussinesq contexts (the assembly reads the
        // temperatures), else on first use of the heat API
        c->heat_ready = false;
        if (c->prm.boussinesq && (rc = heat_alloc(c))) return rc;
        if (c->prm.precision == PFG_PREC_MIXED && (rc = mx_alloc(c))) return rc;
    } else {
        if ((rc = wc_alloc(c))) return rc;
        c->heat_ready = false;  // BoussinesqWC: the temperatures restart at zero with the mesh
        if (c->prm.boussinesq && (rc = heat_alloc(c))) return rc;
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->has_mesh = true;
    return PFG_OK;
}

namespace {
// New node states from the old ones: a copy for one source, the mean in source order for
// several (the centroid node of Mesh::addNodes, Mesh.cpp:59-67).  One thread per (field, node).
__global__ void k_remap(int n_new, int nf, int n_old, const double* __restrict__ old, const int* __restrict__ origin,
                        int width, double* __restrict__ out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n_new * nf) return;
    const int f = (int)(t / n_new), j = (int)(t % n_new);
    const int* o = origin + (size_t)j * width;
    double s = old[(size_t)f * n_old + o[0]];
    int cnt = 1;
    for (int k = 1; k < width && o[k] >= 0; ++k, ++cnt) s += old[(size_t)f * n_old + o[k]];
    out[(size_t)f * n_new + j] = cnt > 1 ? s / cnt : s;
}
}  // namespace

PFG_API int pfg_upload_mesh_remap(pfg_ctx* c, int32_t n_nodes, const double* pos, const uint8_t* flags,
                                  int32_t n_elems, const int32_t* conn, const int32_t* origin, int32_t width) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG)
        return fail(c, PFG_ERR_UNSUPPORTED, "pfg_upload_mesh_remap: incompressible contexts only");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "pfg_upload_mesh_remap: no previous mesh");
    if (!origin || width < 1 || width > 4 || n_nodes <= 0)
        return fail(c, PFG_ERR_INVALID, "pfg_upload_mesh_remap: invalid origin table");
    const int n_old = c->N, nf = c->dim + 1;
    for (int j = 0; j < n_nodes; ++j)
        for (int k = 0; k < width; ++k) {
            const int v = origin[(size_t)j * width + k];
            if ((k == 0 && (v < 0 || v >= n_old)) || v >= n_old || (k > 0 && v < -1))
                return fail(c, PFG_ERR_INVALID, "origin of node %d: %d out of range", j, v);
        }
    // the old states (and temperatures) survive the upload in a scratch buffer
    const bool heat = c->heat_ready;
    const size_t old_n = (size_t)(nf + (heat ? 1 : 0)) * n_old;
    DBuf keep{}, org{};
    auto done = [&](int r) {
        cudaStreamSynchronize(c->stream);
        c->bytes_in_use -= keep.cap + org.cap;
        release(keep);
        release(org);
        return r;
    };
    if ((rc = ensure(c, keep, sizeof(double) * old_n)) ||
        (rc = ensure(c, org, sizeof(int) * (size_t)n_nodes * width)))
        return done(rc);
    if (cudaMemcpyAsync(keep.p, c->q.p, sizeof(double) * nf * n_old, cudaMemcpyDeviceToDevice, c->stream) ||
        (heat && cudaMemcpyAsync(ptr<double>(keep) + (size_t)nf * n_old, c->heat_t.p, sizeof(double) * n_old,
                                 cudaMemcpyDeviceToDevice, c->stream)) ||
        cudaMemcpyAsync(org.p, origin, sizeof(int) * (size_t)n_nodes * width, cudaMemcpyHostToDevice, c->stream))
        return done(fail(c, PFG_ERR_CUDA, "pfg_upload_mesh_remap: copy failed"));
    if ((rc = pfg_upload_mesh(c, n_nodes, pos, flags, n_elems, conn))) return done(rc);
    const long long nt = (long long)n_nodes * nf;
    k_remap<<<div_up(nt, BLOCK), BLOCK, 0, c->stream>>>(n_nodes, nf, n_old, ptr<double>(keep), ptr<int>(org), width,
                                                        ptr<double>(c->q));
    if (heat) {
        if ((rc = heat_alloc(c))) return done(rc);
        k_remap<<<div_up(n_nodes, BLOCK), BLOCK, 0, c->stream>>>(n_nodes, 1, n_old, ptr<double>(keep) + (size_t)nf * n_old,
                                                                 ptr<int>(org), width, ptr<double>(c->heat_t));
    }
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
        return done(fail(c, PFG_ERR_CUDA, "pfg_upload_mesh_remap: remap failed"));
    return done(PFG_OK);
}

PFG_API int pfg_upload_facets(pfg_ctx* c, int32_t n_facets, const int32_t* facets, const int32_t* facet_elm) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (n_facets < 0 || n_facets >= (1 << 29) || (n_facets > 0 && (!facets || !facet_elm)))
        return fail(c, PFG_ERR_INVALID, "pfg_upload_facets: invalid count or null pointers");
    const int dim = c->dim, npe = c->npe, N = c->N, E = c->E, F = n_facets;
    // the facet rule of the kind: any node on the free surface (m_applyBCPSPG,
    // MomContEquationPSPG.inl:163-174) or all of them (Facet::isOnFreeSurface, Facet.cpp:249-255)
    const bool any_node = c->prm.kind == PFG_KIND_INCOMP_PSPG;
    std::vector<uint8_t> use(F, 0);
    std::vector<int> cnt((size_t)N + 1, 0);
    for (int f = 0; f < F; ++f) {
        const int e = facet_elm[f];
        if (e < 0 || e >= E) return fail(c, PFG_ERR_INVALID, "facet %d: element %d out of range", f, e);
        int on_fs = 0;
        for (int k = 0; k < dim; ++k) {
            const int v = facets[(size_t)k * F + f];
            bool in = false;
            for (int i = 0; i < npe; ++i) in |= c->h_conn[(size_t)i * E + e] == v;
            if (!in) return fail(c, PFG_ERR_INVALID, "facet %d: node %d is not a node of element %d", f, v, e);
            on_fs += (c->h_flags[v] & F_FREE_SURFACE) ? 1 : 0;
        }
        use[f] = any_node ? on_fs > 0 : on_fs == dim;
        if (use[f])
            for (int i = 0; i < npe; ++i) cnt[c->h_conn[(size_t)i * E + e]]++;
    }
    // listed nodes (ascending) with their entries in ascending facet order (the order the
    // reference adds them)
    std::vector<int> nodes, nf_ptr(1, 0), slot((size_t)N, -1);
    for (int n = 0; n < N; ++n)
        if (cnt[n]) {
            slot[n] = nf_ptr.back();
            nodes.push_back(n);
            nf_ptr.push_back(nf_ptr.back() + cnt[n]);
        }
    std::vector<int> nf_ent(std::max(nf_ptr.back(), 1));
    for (int f = 0; f < F; ++f)
        if (use[f])
            for (int i = 0; i < npe; ++i) nf_ent[slot[c->h_conn[(size_t)i * E + facet_elm[f]]]++] = f * 4 + i;
    const size_t nf = std::max<size_t>((size_t)F, 1), nn = std::max<size_t>(nodes.size(), 1);
    if ((rc = ensure(c, c->fc_nodes, sizeof(int) * dim * nf)) || (rc = ensure(c, c->fc_elem, sizeof(int) * nf)) ||
        (rc = ensure(c, c->nf_nodes, sizeof(int) * nn)) || (rc = ensure(c, c->nf_ptr, sizeof(int) * (nn + 1))) ||
        (rc = ensure(c, c->nf_ent, sizeof(int) * nf_ent.size())) ||
        (rc = ensure(c, c->fst_force, sizeof(double) * dim * (size_t)N)))
        return rc;
    if (F) {
        PFG_CUDA(c, cudaMemcpyAsync(c->fc_nodes.p, facets, sizeof(int) * dim * (size_t)F, cudaMemcpyHostToDevice, c->stream));
        PFG_CUDA(c, cudaMemcpyAsync(c->fc_elem.p, facet_elm, sizeof(int) * (size_t)F, cudaMemcpyHostToDevice, c->stream));
    }
    if (!nodes.empty())
        PFG_CUDA(c, cudaMemcpyAsync(c->nf_nodes.p, nodes.data(), sizeof(int) * nodes.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->nf_ptr.p, nf_ptr.data(), sizeof(int) * nf_ptr.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->nf_ent.p, nf_ent.data(), sizeof(int) * nf_ent.size(), cudaMemcpyHostToDevice, c->stream));
    // nodes outside the list keep a zero force
    PFG_CUDA(c, cudaMemsetAsync(c->fst_force.p, 0, sizeof(double) * dim * (size_t)N, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->F = F;
    c->n_fst_nodes = (int)nodes.size();
    c->has_facets = true;
    c->h_facets.assign(facets, facets + (size_t)dim * F);
    c->h_facet_elm.assign(facet_elm, facet_elm + F);
    c->has_heat_q = false;  // flux vectors are per facet: a new facet list needs new ones
    c->heat_facets_dirty = true;
    // captured WC step graphs hold the previous facet arguments
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT) wc_release_graphs(c);
    return PFG_OK;
}

// ---- heat equation -----------------------------------------------------------------------

namespace {
int check_heat(pfg_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG && !c->prm.boussinesq)
        return fail(c, PFG_ERR_UNSUPPORTED, "the heat equation needs an incompressible or a BoussinesqWC context");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    return c->heat_ready ? PFG_OK : heat_alloc(c);
}
}  // namespace

PFG_API int pfg_set_temperature(pfg_ctx* c, const double* T) {
    int rc = check_heat(c);
    if (rc) return rc;
    if (!T) return fail(c, PFG_ERR_INVALID, "null temperatures");
    PFG_CUDA(c, cudaMemcpyAsync(c->heat_t.p, T, sizeof(double) * c->N, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_get_temperature(pfg_ctx* c, double* T) {
    int rc = check_heat(c);
    if (rc) return rc;
    if (!T) return fail(c, PFG_ERR_INVALID, "null temperatures");
    PFG_CUDA(c, cudaMemcpyAsync(T, c->heat_t.p, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_heat_set_bc(pfg_ctx* c, const uint8_t* flags, const double* t_dirichlet) {
    int rc = check_heat(c);
    if (rc) return rc;
    if (!flags) return fail(c, PFG_ERR_INVALID, "null heat flags");
    const int N = c->N;
    bool any_t = false;
    for (int n = 0; n < N; ++n) {
        if (flags[n] & ~(PFG_HEAT_T | PFG_HEAT_Q | PFG_HEAT_QH | PFG_HEAT_QR))
            return fail(c, PFG_ERR_INVALID, "node %d: unknown heat flag bits 0x%x", n, flags[n]);
        // the reference rejects a boundary with both a T and a flux condition (Solver.cpp:160-162)
        if ((flags[n] & PFG_HEAT_T) && (flags[n] & (PFG_HEAT_Q | PFG_HEAT_QH | PFG_HEAT_QR)))
            return fail(c, PFG_ERR_INVALID, "node %d: both a T and a flux heat condition", n);
        any_t |= (flags[n] & PFG_HEAT_T) != 0;
    }
    if (any_t && !t_dirichlet) return fail(c, PFG_ERR_INVALID, "Dirichlet heat nodes need t_dirichlet");
    c->h_heat_flags.assign(flags, flags + N);
    c->heat_facets_dirty = true;
    PFG_CUDA(c, cudaMemcpyAsync(c->heat_flags.p, flags, N, cudaMemcpyHostToDevice, c->stream));
    if (t_dirichlet)
        PFG_CUDA(c, cudaMemcpyAsync(c->heat_tbc.p, t_dirichlet, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->has_heat_bc = true;
    return PFG_OK;
}

PFG_API int pfg_heat_set_flux(pfg_ctx* c, const double* q_gp) {
    int rc = check_heat(c);
    if (rc) return rc;
    c->heat_facets_dirty = true;  // the Q requirement is checked with the lists
    if (!q_gp) {
        c->has_heat_q = false;
        return PFG_OK;
    }
    if (!c->has_facets) return fail(c, PFG_ERR_STATE, "pfg_heat_set_flux: call pfg_upload_facets first");
    const size_t n = (size_t)std::max(c->F, 1) * 3 * c->dim;
    if ((rc = ensure(c, c->heat_q, sizeof(double) * n))) return rc;
    if (c->F)
        PFG_CUDA(c, cudaMemcpyAsync(c->heat_q.p, q_gp, sizeof(double) * (size_t)c->F * 3 * c->dim,
                                    cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->has_heat_q = true;
    return PFG_OK;
}

PFG_API int pfg_heat_step(pfg_ctx* c, double dt, pfg_step_status* st) {
    int rc = check_heat(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG)
        return fail(c, PFG_ERR_UNSUPPORTED, "BoussinesqWC runs its heat step inside pfg_wc_step");
    if (!st) return fail(c, PFG_ERR_INVALID, "null status");
    if (!(dt > 0)) return fail(c, PFG_ERR_INVALID, "dt must be > 0");
    if (!(c->prm.heat_cv * c->prm.rho > 0) || !(c->prm.heat_k >= 0))
        return fail(c, PFG_ERR_INVALID, "heat: needs cv rho > 0 and k >= 0");
    bool flux = (c->prm.heat_fs_flags & (PFG_HEAT_Q | PFG_HEAT_QH | PFG_HEAT_QR)) != 0;
    for (uint8_t f : c->h_heat_flags) flux |= (f & (PFG_HEAT_Q | PFG_HEAT_QH | PFG_HEAT_QR)) != 0;
    if (flux && !c->has_facets) return fail(c, PFG_ERR_STATE, "heat flux conditions need pfg_upload_facets");
    std::memset(st, 0, sizeof(*st));
    if ((rc = heat_build_facets(c))) return rc;
    return heat_step(c, dt, st);
}

PFG_API int pfg_set_states(pfg_ctx* c, const double* states) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!states) return fail(c, PFG_ERR_INVALID, "null states");
    if (c->prm.kind == PFG_KIND_INCOMP_PSPG) {
        PFG_CUDA(c, cudaMemcpyAsync(c->q.p, states, sizeof(double) * c->R, cudaMemcpyHostToDevice, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        return PFG_OK;
    }
    return wc_set_states(c, states);
}

PFG_API int pfg_get_states(pfg_ctx* c, double* states) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!states) return fail(c, PFG_ERR_INVALID, "null states");
    if (c->prm.kind == PFG_KIND_INCOMP_PSPG) {
        PFG_CUDA(c, cudaMemcpyAsync(states, c->q.p, sizeof(double) * c->R, cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        return PFG_OK;
    }
    return wc_get_states(c, states);
}

PFG_API int pfg_get_positions(pfg_ctx* c, double* pos) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!pos) return fail(c, PFG_ERR_INVALID, "null positions");
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT && (rc = wc_sync_positions(c))) return rc;
    PFG_CUDA(c, cudaMemcpyAsync(pos, c->pos.p, sizeof(double) * c->dim * c->N, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_set_positions(pfg_ctx* c, const double* pos) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!pos) return fail(c, PFG_ERR_INVALID, "null positions");
    const size_t bytes = sizeof(double) * c->dim * c->N;
    PFG_CUDA(c, cudaMemcpyAsync(c->pos.p, pos, bytes, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->pos_save.p, pos, bytes, cudaMemcpyHostToDevice, c->stream));
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT && c->prm.precision == PFG_PREC_MIXED && (rc = wcm_positions_in(c)))
        return rc;
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_get_flags(pfg_ctx* c, uint8_t* flags) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!flags) return fail(c, PFG_ERR_INVALID, "null flags");
    PFG_CUDA(c, cudaMemcpyAsync(flags, c->flags.p, c->N, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_set_dirichlet(pfg_ctx* c, int32_t n, const int32_t* nodes, const double* values) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (n < 0 || (n > 0 && (!nodes || !values))) return fail(c, PFG_ERR_INVALID, "pfg_set_dirichlet: bad arguments");
    if (n == 0) return PFG_OK;
    for (int i = 0; i < n; ++i)
        if (nodes[i] < 0 || nodes[i] >= c->N) return fail(c, PFG_ERR_INVALID, "Dirichlet node %d out of range", nodes[i]);
    DBuf tmp;
    const size_t nb = sizeof(int) * n, vb = sizeof(double) * c->dim * n;
    if ((rc = ensure(c, tmp, nb + vb + 256))) return rc;
    char* base = ptr<char>(tmp);
    int* dn = reinterpret_cast<int*>(base);
    double* dv = reinterpret_cast<double*>(base + ((nb + 255) & ~(size_t)255));
    cudaError_t e = cudaMemcpyAsync(dn, nodes, nb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dv, values, vb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        k_scatter_dirichlet<<<div_up(n, BLOCK), BLOCK, 0, c->stream>>>(n, dn, dv, c->N, c->dim, ptr<double>(c->vbc));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    c->bytes_in_use -= tmp.cap;
    release(tmp);
    if (e != cudaSuccess) return cuda_fail(c, e, "pfg_set_dirichlet");
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT) return wc_dirichlet_changed(c);
    return PFG_OK;
}

PFG_API int pfg_picard_step(pfg_ctx* c, double dt, pfg_step_status* st) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG) return fail(c, PFG_ERR_STATE, "context is not incompressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if ((rc = check_facets(c))) return rc;
    if (!(dt > 0) || !st) return fail(c, PFG_ERR_INVALID, "pfg_picard_step: dt must be > 0 and status non-null");
    if (c->prm.precision == PFG_PREC_MIXED) {
        if (c->n_inst != 1) return fail(c, PFG_ERR_STATE, "context holds %d instances: use pfg_picard_step_batch", c->n_inst);
        return mx_picard_step(c, &dt, st);
    }
    if (c->prm.frac_step) return fs_picard_step(c, dt, st);
    return picard_step(c, dt, st);
}

PFG_API int pfg_device_bytes(const pfg_ctx* c, size_t* bytes) {
    if (!c || !bytes) return PFG_ERR_INVALID;
    *bytes = c->bytes_in_use;
    return PFG_OK;
}

PFG_API int pfg_set_instances(pfg_ctx* c, int32_t n_inst, const int32_t* node_offsets, const double* rho,
                              const double* mu) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.precision != PFG_PREC_MIXED)
        return fail(c, PFG_ERR_STATE, "instances need a context in mixed precision");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (n_inst <= 0 || !node_offsets || !rho || !mu) return fail(c, PFG_ERR_INVALID, "pfg_set_instances: bad arguments");
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT)
        for (int i = 0; i < n_inst; ++i)
            if (rho[i] != c->prm.rho_star)
                return fail(c, PFG_ERR_UNSUPPORTED, "weakly compressible instances share rho* (instance %d)", i);
    if (node_offsets[0] != 0 || node_offsets[n_inst] != c->N)
        return fail(c, PFG_ERR_INVALID, "node offsets must start at 0 and end at the node count %d", c->N);
    for (int i = 0; i < n_inst; ++i) {
        if (node_offsets[i + 1] < node_offsets[i]) return fail(c, PFG_ERR_INVALID, "node offsets must not decrease");
        if (!(rho[i] > 0) || !(mu[i] >= 0)) return fail(c, PFG_ERR_INVALID, "instance %d: rho must be > 0, mu >= 0", i);
    }
    // every element must stay inside one instance
    std::vector<int> conn((size_t)c->npe * c->E);
    if (c->E) {
        PFG_CUDA(c, cudaMemcpyAsync(conn.data(), c->conn.p, sizeof(int) * conn.size(), cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    auto inst_of = [&](int n) {
        return (int)(std::upper_bound(node_offsets, node_offsets + n_inst + 1, n) - node_offsets) - 1;
    };
    for (int e = 0; e < c->E; ++e) {
        const int i0 = inst_of(conn[e]);
        for (int k = 1; k < c->npe; ++k)
            if (inst_of(conn[(size_t)k * c->E + e]) != i0)
                return fail(c, PFG_ERR_INVALID, "element %d joins nodes of two instances", e);
    }
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT) {
        if (c->has_facets) return fail(c, PFG_ERR_UNSUPPORTED, "batched weakly compressible steps without facets");
        return wcm_set_instances(c, n_inst, node_offsets, mu);
    }
    return mx_set_instances(c, n_inst, node_offsets, rho, mu);
}

PFG_API int pfg_picard_step_batch(pfg_ctx* c, const double* dt, pfg_step_status* st) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG || c->prm.precision != PFG_PREC_MIXED)
        return fail(c, PFG_ERR_STATE, "batched steps need an incompressible context in mixed precision");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if ((rc = check_facets(c))) return rc;
    if (!dt || !st) return fail(c, PFG_ERR_INVALID, "pfg_picard_step_batch: null arguments");
    for (int i = 0; i < c->n_inst; ++i)
        if (!(dt[i] > 0)) return fail(c, PFG_ERR_INVALID, "instance %d: dt must be > 0", i);
    return mx_picard_step(c, dt, st);
}

PFG_API int pfg_wc_step(pfg_ctx* c, double dt, int32_t nsteps, pfg_step_status* st) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_WC_CDS_DPDT) return fail(c, PFG_ERR_STATE, "context is not weakly compressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if ((rc = check_facets(c))) return rc;
    if (nsteps < 0 || !st) return fail(c, PFG_ERR_INVALID, "pfg_wc_step: bad arguments");
    return wc_steps(c, dt, nsteps, st);
}

PFG_API int pfg_wc_step_batch(pfg_ctx* c, double dt, int32_t nsteps, pfg_step_status* st) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_WC_CDS_DPDT) return fail(c, PFG_ERR_STATE, "context is not weakly compressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (nsteps < 0 || !st) return fail(c, PFG_ERR_INVALID, "pfg_wc_step_batch: bad arguments");
    c->wc_pending = 0;
    if ((rc = wc_enqueue(c, dt, nsteps))) return rc;
    return wc_sync_batch(c, st);
}

PFG_API int pfg_wc_step_async(pfg_ctx* c, double dt, int32_t nsteps) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_WC_CDS_DPDT) return fail(c, PFG_ERR_STATE, "context is not weakly compressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if ((rc = check_facets(c))) return rc;
    if (nsteps < 0) return fail(c, PFG_ERR_INVALID, "pfg_wc_step_async: nsteps < 0");
    return wc_enqueue(c, dt, nsteps);
}

PFG_API int pfg_synchronize(pfg_ctx* c, pfg_step_status* st) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!st) return fail(c, PFG_ERR_INVALID, "null status");
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT && c->has_mesh) return wc_sync(c, st);
    std::memset(st, 0, sizeof(*st));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_get_stream(pfg_ctx* c, void** stream) {
    if (!c || !stream) return PFG_ERR_INVALID;
    *stream = (void*)c->stream;
    return PFG_OK;
}

PFG_API int pfg_next_dt(pfg_ctx* c, double* dt) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_WC_CDS_DPDT) return fail(c, PFG_ERR_STATE, "context is not weakly compressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!dt) return fail(c, PFG_ERR_INVALID, "null dt");
    return wc_next_dt(c, dt);
}

PFG_API int pfg_set_time(pfg_ctx* c, double time, double next_dt) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_WC_CDS_DPDT) return fail(c, PFG_ERR_STATE, "context is not weakly compressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    return wc_set_time(c, time, next_dt);
}

PFG_API int pfg_volume(pfg_ctx* c, double* v) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!v) return fail(c, PFG_ERR_INVALID, "null output");
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT && (rc = wc_sync_positions(c))) return rc;
    return volume(c, v);
}

PFG_API int pfg_mass(pfg_ctx* c, double* m) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!m) return fail(c, PFG_ERR_INVALID, "null output");
    if (c->prm.kind == PFG_KIND_INCOMP_PSPG) return volume(c, m);
    return wc_mass(c, m);
}

PFG_API int pfg_tip(pfg_ctx* c, int32_t coord, int32_t want_max, double* v) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!v || coord < 0 || coord >= c->dim) return fail(c, PFG_ERR_INVALID, "bad coordinate");
    if (c->prm.kind == PFG_KIND_WC_CDS_DPDT && (rc = wc_sync_positions(c))) return rc;
    return tip(c, coord, want_max, v);
}

PFG_API int pfg_pspg_assemble(pfg_ctx* c, double dt, const double* q_iter, const double* q_prev, int32_t apply_bc) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG) return fail(c, PFG_ERR_STATE, "context is not incompressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if ((rc = check_facets(c))) return rc;
    if (!(dt > 0)) return fail(c, PFG_ERR_INVALID, "dt must be > 0");
    double* kv = ptr<double>(c->kv);
    const size_t R = c->R;
    // stage host vectors in Krylov workspace slots 8 and 9
    const double* di = ptr<double>(c->q);
    const double* dp = ptr<double>(c->q);
    if (q_iter) {
        PFG_CUDA(c, cudaMemcpyAsync(kv + 8 * R, q_iter, sizeof(double) * R, cudaMemcpyHostToDevice, c->stream));
        di = kv + 8 * R;
    }
    if (q_prev) {
        PFG_CUDA(c, cudaMemcpyAsync(kv + 9 * R, q_prev, sizeof(double) * R, cudaMemcpyHostToDevice, c->stream));
        dp = kv + 9 * R;
    }
    rc = pspg_assemble(c, dt, di, dp, apply_bc != 0);
    if (rc) return rc;
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_get_csr(pfg_ctx* c, int32_t* n_rows, int64_t* nnz, int64_t* row_ptr, int32_t* col_idx,
                        double* values, double* rhs) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG) return fail(c, PFG_ERR_STATE, "context is not incompressible");
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (n_rows) *n_rows = c->R;
    if (nnz) *nnz = c->nnz;
    if (row_ptr) {
        std::vector<int> tmp(c->R + 1);
        PFG_CUDA(c, cudaMemcpyAsync(tmp.data(), c->row_ptr.p, sizeof(int) * (c->R + 1), cudaMemcpyDeviceToHost,
                                    c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int i = 0; i <= c->R; ++i) row_ptr[i] = tmp[i];
    }
    if (col_idx)
        PFG_CUDA(c, cudaMemcpyAsync(col_idx, c->col.p, sizeof(int) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
    if (values || rhs) {
        if (!c->has_system) return fail(c, PFG_ERR_STATE, "no assembled system");
        if (values)
            PFG_CUDA(c, cudaMemcpyAsync(values, c->val.p, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
        if (rhs) PFG_CUDA(c, cudaMemcpyAsync(rhs, c->rhs.p, sizeof(double) * c->R, cudaMemcpyDeviceToHost, c->stream));
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

PFG_API int pfg_get_geometry(pfg_ctx* c, double* detJ, double* invJ) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->has_mesh) return fail(c, PFG_ERR_STATE, "no mesh uploaded");
    if (!detJ || !invJ) return fail(c, PFG_ERR_INVALID, "null output");
    DBuf tmp;
    if ((rc = ensure(c, tmp, sizeof(double) * 10 * (size_t)std::max(c->E, 1)))) return rc;
    double* d = ptr<double>(tmp);
    rc = compute_geometry(c, d, d + c->E);
    cudaError_t e = cudaSuccess;
    if (!rc) e = cudaMemcpyAsync(detJ, d, sizeof(double) * c->E, cudaMemcpyDeviceToHost, c->stream);
    if (!rc && e == cudaSuccess)
        e = cudaMemcpyAsync(invJ, d + c->E, sizeof(double) * 9 * c->E, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    c->bytes_in_use -= tmp.cap;
    release(tmp);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(c, e, "pfg_get_geometry");
    return PFG_OK;
}

PFG_API int pfg_linear_solve(pfg_ctx* c, double* x, int32_t* iterations, double* res) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->prm.kind != PFG_KIND_INCOMP_PSPG) return fail(c, PFG_ERR_STATE, "context is not incompressible");
    if (!c->has_system) return fail(c, PFG_ERR_STATE, "no assembled system");
    if (!x) return fail(c, PFG_ERR_INVALID, "null x");
    double* kv = ptr<double>(c->kv);
    double* dx = kv + 8 * (size_t)c->R;
    PFG_CUDA(c, cudaMemcpyAsync(dx, x, sizeof(double) * c->R, cudaMemcpyHostToDevice, c->stream));
    int it = 0;
    double r = 0;
    rc = bicgstab(c, dx, &it, &r);
    if (rc) return rc;
    PFG_CUDA(c, cudaMemcpyAsync(x, dx, sizeof(double) * c->R, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (iterations) *iterations = it;
    if (res) *res = r;
    return PFG_OK;
}

}  // extern "C"
