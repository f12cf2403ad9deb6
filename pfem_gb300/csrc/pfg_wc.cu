// Weakly compressible explicit step (CDS_dpdt with the Tait-Murnaghan equation of state).
//
// Reference: SolverWCompNewton::m_solveWCompNewtonNoT (WCompNewton/Solver.cpp:236-276),
// ContEqWCompNewton::m_buildSystemdpdt/m_applyBCdpdt/solve (ContEquation.inl:123-169,
// :334-413), MomEqWCompNewton::m_buildSystem/m_applyBC/solve (MomEquation.inl:201-374) and
// SolverWCompNewton::computeNextDT (Solver.cpp:192-234).
//
// One step is five kernels (six with the CFL time step):
//   predict   (node)    v1/2 = v + dt/2 a ; x += dt v1/2 for non-fixed nodes
//   cont_elem (element) lumped mass and F0e = -dt D(K0+K0'p) v + M p   (Meduri) per element node
//   cont_node (node)    gather over the node's elements in element order -> p, rho (Tait)
//   mom_elem  (element) lumped rho-mass and FTot = -K v + D^T p + F(rho g) per element node
//   mom_node  (node)    gather -> a = F / M (with BCs), v = v1/2 + dt/2 a
//   dt        (element) min over elements of sc^2 h^2 / max(u^2, c^2, 4 alpha^2/h^2) -> next dt
// The element->node gathers sum in ascending element order, the order of the reference's
// serial scatter loops, so results do not depend on scheduling.  The state is a template
// type (double for the plain form, float for the mixed form); positions and element geometry
// stay FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

struct WcConst {
    double K0, K0p, rho_star, mu, sc, max_dt;
    double g[3];
    int meduri;
    int ng;
    double w[4];
    double N[4][4];
    double MM[4][4];
    double s[4];
    double refSize;
    double mu_sum;
};

WcConst make_const(pfg_ctx* c) {
    const GaussConst gc = gauss_const(c->dim);
    WcConst k{};
    k.K0 = c->prm.K0;
    k.K0p = c->prm.K0p;
    k.rho_star = c->prm.rho_star;
    k.mu = c->prm.mu;
    k.sc = c->prm.security_coeff;
    k.max_dt = c->prm.max_dt;
    for (int f = 0; f < 3; ++f) k.g[f] = c->prm.gravity[f];
    k.meduri = c->prm.meduri;
    k.ng = gc.n;
    for (int q = 0; q < 4; ++q) {
        k.w[q] = gc.w[q];
        k.s[q] = gc.s[q];
        for (int i = 0; i < 4; ++i) {
            k.N[q][i] = gc.N[q][i];
            k.MM[q][i] = gc.MM[q][i];
        }
    }
    k.refSize = gc.refSize;
    k.mu_sum = 0;
    for (int q = 0; q < gc.n; ++q) k.mu_sum += c->prm.mu * gc.w[q];
    return k;
}

// slots of ctx->wc_dt (doubles)
enum : int { T_DT = 0, T_TIME = 1, T_MIN = 2, T_TICKET = 3 };

template <int DIM, class T>
__global__ void k_wc_predict(int N, const uint8_t* __restrict__ flags, T* __restrict__ s, double* __restrict__ pos,
                             double* __restrict__ tdt) {
    const double dt = tdt[T_DT];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n == 0) tdt[T_TIME] += dt;  // Problem::updateTime with the step's dt
    if (n >= N) return;
    const bool fixed = flags[n] & F_FIXED;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        T* v = s + (size_t)d * N;
        const T* a = s + (size_t)(DIM + 2 + d) * N;
        const T vh = v[n] + (T)(0.5 * dt) * a[n];
        v[n] = vh;
        if (!fixed) pos[(size_t)d * N + n] += (double)vh * dt;
    }
}

template <int DIM, class T>
__global__ void __launch_bounds__(BLOCK) k_wc_cont_elem(int E, int N, const int* __restrict__ conn,
                                                        const double* __restrict__ pos, const T* __restrict__ s,
                                                        const double* __restrict__ tdt, WcConst k,
                                                        T* __restrict__ el) {
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double dt = tdt[T_DT];
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    double G[DIM][NPE];
    grad_n<DIM>(g, G);
    const double ae = g.detJ * k.refSize;
    double P[NPE];
    double divv = 0;
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        P[j] = (double)s[(size_t)DIM * N + nd[j]];
#pragma unroll
        for (int f = 0; f < DIM; ++f) divv += G[f][j] * (double)s[(size_t)f * N + nd[j]];
    }
    // sum_g w_g (K0 + K0' p(g)) N_i(g)
    double swn[NPE];
#pragma unroll
    for (int i = 0; i < NPE; ++i) swn[i] = 0;
    for (int q = 0; q < k.ng; ++q) {
        double pg = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) pg += k.N[q][j] * P[j];
        const double fac = (k.K0 + k.K0p * pg) * k.w[q];
#pragma unroll
        for (int i = 0; i < NPE; ++i) swn[i] += fac * k.N[q][i];
    }
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        double lumped = 0, mp = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            const double mij = k.MM[i][j] * ae;
            lumped += mij;
            mp += mij * P[j];
        }
        const double dv = ae * swn[i] * divv;
        const double f0 = -dt * dv + (k.meduri ? mp : lumped * P[i]);
        el[(size_t)i * E + e] = (T)lumped;
        el[(size_t)(NPE + i) * E + e] = (T)f0;
    }
}

template <int DIM, class T>
__global__ void k_wc_cont_node(int N, int E, const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                               const uint8_t* __restrict__ ne_loc, const uint8_t* __restrict__ flags,
                               const T* __restrict__ el, WcConst k, T* __restrict__ s) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double m = 0, f0 = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q], i = ne_loc[q];
        m += (double)el[(size_t)i * E + e];
        f0 += (double)el[(size_t)(NPE + i) * E + e];
    }
    double inv = 1 / m;
    if (flags[n] & F_FREE) {  // m_applyBCdpdt (ContEquation.inl:343-348)
        f0 = 0;
        inv = 1;
    }
    const double p = inv * f0;
    const double rho = pow((k.K0p / k.K0) * p + 1, 1 / k.K0p) * k.rho_star;
    s[(size_t)DIM * N + n] = (T)p;
    s[(size_t)(DIM + 1) * N + n] = (T)rho;
}

template <int DIM, class T>
__global__ void __launch_bounds__(BLOCK) k_wc_mom_elem(int E, int N, const int* __restrict__ conn,
                                                       const double* __restrict__ pos, const T* __restrict__ s,
                                                       WcConst k, T* __restrict__ el) {
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    double G[DIM][NPE];
    grad_n<DIM>(g, G);
    const double ae = g.detJ * k.refSize;
    double P[NPE], Rh[NPE], V[DIM][NPE];
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        P[j] = (double)s[(size_t)DIM * N + nd[j]];
        Rh[j] = (double)s[(size_t)(DIM + 1) * N + nd[j]];
#pragma unroll
        for (int f = 0; f < DIM; ++f) V[f][j] = (double)s[(size_t)f * N + nd[j]];
    }
    // sum_g w rho(g) N_i(g) N_j(g)  and  sum_g w rho(g) N_i(g)
    double mt[NPE][NPE], fr[NPE];
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        fr[i] = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) mt[i][j] = 0;
    }
    for (int q = 0; q < k.ng; ++q) {
        double rg = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) rg += k.N[q][j] * Rh[j];
        const double fw = rg * k.w[q];
#pragma unroll
        for (int i = 0; i < NPE; ++i) {
            fr[i] += fw * k.N[q][i];
#pragma unroll
            for (int j = 0; j < NPE; ++j) mt[i][j] += fw * k.N[q][i] * k.N[q][j];
        }
    }
    // sum_j s_j p_j (pressure term D^T p: |e| dN_i/dx_f sum_j s_j p_j)
    double sp = 0;
#pragma unroll
    for (int j = 0; j < NPE; ++j) sp += k.s[j] * P[j];
    const double kf = ae * k.mu_sum;
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        double lumped = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) lumped += mt[i][j] * ae;
        el[(size_t)i * E + e] = (T)lumped;
#pragma unroll
        for (int f1 = 0; f1 < DIM; ++f1) {
            // (K v)(i f1) with Ddev = [4/3 -2/3 ..; ..] (normal) and 1 (shear), MomEquation.inl:63-83
            double kv = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) {
                double dot = 0;
#pragma unroll
                for (int f = 0; f < DIM; ++f) dot += G[f][i] * G[f][j];
#pragma unroll
                for (int f2 = 0; f2 < DIM; ++f2) {
                    const double kk = (f1 == f2 ? dot : 0.0) + G[f2][i] * G[f1][j] - (2.0 / 3.0) * G[f1][i] * G[f2][j];
                    kv += kf * kk * V[f2][j];
                }
            }
            const double dtp = ae * G[f1][i] * sp;
            const double F = ae * fr[i] * k.g[f1];
            el[(size_t)(NPE + f1 * NPE + i) * E + e] = (T)(-kv + dtp + F);
        }
    }
}

template <int DIM, class T>
__global__ void k_wc_mom_node(int N, int E, const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                              const uint8_t* __restrict__ ne_loc, const uint8_t* __restrict__ flags,
                              const T* __restrict__ el, const double* __restrict__ vbc, const double* __restrict__ tdt,
                              WcConst k, T* __restrict__ s) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double dt = tdt[T_DT];
    double m = 0, F[DIM];
#pragma unroll
    for (int f = 0; f < DIM; ++f) F[f] = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q], i = ne_loc[q];
        m += (double)el[(size_t)i * E + e];
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] += (double)el[(size_t)(NPE + f * NPE + i) * E + e];
    }
    double inv = 1 / m;
    const uint8_t fl = flags[n];
    if ((fl & F_FREE) && !(fl & F_BOUND)) {  // free fall (MomEquation.inl:347-354)
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] = k.g[f];
        inv = 1;
    } else if ((fl & F_BOUND) && (fl & F_DIRICHLET)) {  // V_bc used as acceleration (:355-371)
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] = vbc[(size_t)f * N + n];
        inv = 1;
    }
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        const double a = inv * F[f];
        T* v = s + (size_t)f * N;
        s[(size_t)(DIM + 2 + f) * N + n] = (T)a;
        v[n] = (T)((double)v[n] + 0.5 * dt * a);
    }
}

// computeNextDT: one thread per element, block min, grid min by the last block.
template <int DIM, class T>
__global__ void __launch_bounds__(BLOCK) k_wc_dt(int E, int N, const int* __restrict__ conn,
                                                 const double* __restrict__ pos, const T* __restrict__ s, WcConst k,
                                                 double* __restrict__ partials, double* __restrict__ tdt) {
    __shared__ double sh[32];
    double best = 1.79769313486231570e308;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        int nd[DIM + 1];
        load_nodes<DIM>(conn, E, e, nd);
        double X[DIM + 1][DIM];
#pragma unroll
        for (int a = 0; a <= DIM; ++a)
#pragma unroll
            for (int d = 0; d < DIM; ++d) X[a][d] = pos[(size_t)d * N + nd[a]];
        Geom<DIM> g;
        compute_geom<DIM>(pos, N, nd, g);
        const double size = g.detJ * k.refSize;
        double he;
        if constexpr (DIM == 2) {  // Element::getRin 2D (Element.cpp:228-241)
            auto dist = [&](int a, int b) {
                const double dx = X[a][0] - X[b][0], dy = X[a][1] - X[b][1];
                return sqrt(dx * dx + dy * dy);
            };
            const double sp = (dist(0, 1) + dist(1, 2) + dist(0, 2)) / 2;
            he = 2 * (size / sp);
        } else {  // Element::getRin 3D (Element.cpp:242-293)
            auto nrm = [&](int a0, int a1, int a2) {
                const double ux = X[a1][0] - X[a0][0], uy = X[a1][1] - X[a0][1], uz = X[a1][2] - X[a0][2];
                const double wx = X[a2][0] - X[a0][0], wy = X[a2][1] - X[a0][1], wz = X[a2][2] - X[a0][2];
                const double cx = uy * wz - uz * wy, cy = uz * wx - ux * wz, cz = ux * wy - uy * wx;
                return sqrt(cx * cx + cy * cy + cz * cz);
            };
            const double sum = nrm(0, 1, 2) + nrm(0, 3, 2) + nrm(0, 1, 3) + nrm(3, 1, 2);
            he = 2 * (6 * size / sum);
        }
        double maxSq = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) {
            const int n = nd[a];
            const double p = (double)s[(size_t)DIM * N + n];
            const double rho = (double)s[(size_t)(DIM + 1) * N + n];
            const double c2 = (k.K0 + k.K0p * p) / rho;
            double u2 = 0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double v = (double)s[(size_t)d * N + n];
                u2 += v * v;
            }
            const double alpha = k.mu / rho;
            maxSq = fmax(fmax(u2, c2), maxSq);
            maxSq = fmax(maxSq, 4 * alpha * alpha / (he * he));
        }
        best = fmin(best, k.sc * k.sc * he * he / maxSq);
    }
    best = block_min<BLOCK>(best, sh);
    __shared__ bool last;
    unsigned* ticket = reinterpret_cast<unsigned*>(tdt + T_TICKET);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = best;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double m = 1.79769313486231570e308;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) m = fmin(m, ((volatile double*)partials)[i]);
    m = block_min<BLOCK>(m, sh);
    if (threadIdx.x == 0) {
        tdt[T_DT] = fmin(sqrt(m), k.max_dt);
        tdt[T_MIN] = m;
        *ticket = 0u;
    }
}

template <int DIM>
__global__ void k_wc_mass(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                          const void* __restrict__ sv, int fp32, double refSize, double* partials, unsigned* ticket,
                          double* out) {
    __shared__ double sh[32];
    double acc = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        int nd[DIM + 1];
        load_nodes<DIM>(conn, E, e, nd);
        Geom<DIM> g;
        compute_geom<DIM>(pos, N, nd, g);
        double mid = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) {
            const size_t k = (size_t)(DIM + 1) * N + nd[a];
            mid += fp32 ? (double)static_cast<const float*>(sv)[k] : static_cast<const double*>(sv)[k];
        }
        mid /= (double)(DIM + 1);
        acc += mid * (g.detJ * refSize);
    }
    grid_sum_last<BLOCK>(acc, partials, ticket, sh, out);
}

template <class T>
__global__ void k_convert_in(size_t n, const double* __restrict__ src, T* __restrict__ dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (T)src[i];
}

template <class T>
__global__ void k_convert_out(size_t n, const T* __restrict__ src, double* __restrict__ dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

bool fp32(pfg_ctx* c) { return c->prm.precision == PFG_PREC_MIXED; }

__global__ void k_set_value(double* p, double v) { *p = v; }

template <int DIM, class T>
int launch_step(pfg_ctx* c, bool adapt, const WcConst& k) {
    const int N = c->N, E = c->E;
    T* s = ptr<T>(c->ws);
    T* el = ptr<T>(c->wc_el);
    double* tdt = ptr<double>(c->wc_dt);
    const int gn = div_up(N, BLOCK), ge = std::max(1, div_up(E, BLOCK));
    prof_begin(c, PH_WC_PREDICT);
    k_wc_predict<DIM, T><<<gn, BLOCK, 0, c->stream>>>(N, ptr<uint8_t>(c->flags), s, ptr<double>(c->pos), tdt);
    prof_end(c, PH_WC_PREDICT);
    if (E > 0) {
        prof_begin(c, PH_WC_CONT_ELEM);
        k_wc_cont_elem<DIM, T><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), s, tdt, k,
                                                            el);
        prof_end(c, PH_WC_CONT_ELEM);
    }
    prof_begin(c, PH_WC_CONT_NODE);
    k_wc_cont_node<DIM, T><<<gn, BLOCK, 0, c->stream>>>(N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem),
                                                        ptr<uint8_t>(c->ne_loc), ptr<uint8_t>(c->flags), el, k, s);
    prof_end(c, PH_WC_CONT_NODE);
    if (E > 0) {
        prof_begin(c, PH_WC_MOM_ELEM);
        k_wc_mom_elem<DIM, T><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), s, k, el);
        prof_end(c, PH_WC_MOM_ELEM);
    }
    prof_begin(c, PH_WC_MOM_NODE);
    k_wc_mom_node<DIM, T><<<gn, BLOCK, 0, c->stream>>>(N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem),
                                                       ptr<uint8_t>(c->ne_loc), ptr<uint8_t>(c->flags), el,
                                                       ptr<double>(c->vbc), tdt, k, s);
    prof_end(c, PH_WC_MOM_NODE);
    if (adapt && E > 0) {
        const int grid = std::min(c->max_grid, ge);
        prof_begin(c, PH_WC_DT);
        k_wc_dt<DIM, T><<<grid, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), s, k,
                                                       ptr<double>(c->red), tdt);
        prof_end(c, PH_WC_DT);
    }
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

template <int DIM, class T>
int dt_only(pfg_ctx* c, const WcConst& k) {
    const int E = c->E;
    if (E == 0) return fail(c, PFG_ERR_STATE, "no elements");
    const int grid = std::min(c->max_grid, div_up(E, BLOCK));
    k_wc_dt<DIM, T><<<grid, BLOCK, 0, c->stream>>>(E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), ptr<T>(c->ws), k,
                                                   ptr<double>(c->red), ptr<double>(c->wc_dt));
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

}  // namespace

int wc_alloc(pfg_ctx* c) {
    const size_t es = fp32(c) ? sizeof(float) : sizeof(double);
    const size_t N = c->N, E = std::max(c->E, 1);
    int rc;
    if ((rc = ensure(c, c->ws, es * (2 * c->dim + 2) * N)) ||
        (rc = ensure(c, c->wc_el, es * (size_t)(c->dim + 1) * c->npe * E)) || (rc = ensure(c, c->wc_dt, 64)))
        return rc;
    PFG_CUDA(c, cudaMemsetAsync(c->ws.p, 0, es * (2 * c->dim + 2) * N, c->stream));
    double h[4] = {c->prm.max_dt, c->host_time, 0.0, 0.0};
    PFG_CUDA(c, cudaMemcpyAsync(c->wc_dt.p, h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_set_states(pfg_ctx* c, const double* h) {
    const size_t n = (size_t)(2 * c->dim + 2) * c->N;
    if (!fp32(c)) {
        PFG_CUDA(c, cudaMemcpyAsync(c->ws.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    } else {
        int rc = ensure(c, c->stage, sizeof(double) * n);
        if (rc) return rc;
        PFG_CUDA(c, cudaMemcpyAsync(c->stage.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        k_convert_in<float><<<std::min(c->max_grid, div_up((long long)n, BLOCK)), BLOCK, 0, c->stream>>>(
            n, ptr<double>(c->stage), ptr<float>(c->ws));
        PFG_CHECK_LAUNCH(c);
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_get_states(pfg_ctx* c, double* h) {
    const size_t n = (size_t)(2 * c->dim + 2) * c->N;
    if (!fp32(c)) {
        PFG_CUDA(c, cudaMemcpyAsync(h, c->ws.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    } else {
        int rc = ensure(c, c->stage, sizeof(double) * n);
        if (rc) return rc;
        k_convert_out<float><<<std::min(c->max_grid, div_up((long long)n, BLOCK)), BLOCK, 0, c->stream>>>(
            n, ptr<float>(c->ws), ptr<double>(c->stage));
        PFG_CHECK_LAUNCH(c);
        PFG_CUDA(c, cudaMemcpyAsync(h, c->stage.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_enqueue(pfg_ctx* c, double dt, int nsteps) {
    const bool adapt = !(dt > 0);
    if (!adapt) {
        k_set_value<<<1, 1, 0, c->stream>>>(ptr<double>(c->wc_dt) + T_DT, dt);
        PFG_CHECK_LAUNCH(c);
    }
    const WcConst k = make_const(c);
    for (int i = 0; i < nsteps; ++i) {
        int rc;
        if (c->dim == 2)
            rc = fp32(c) ? launch_step<2, float>(c, adapt, k) : launch_step<2, double>(c, adapt, k);
        else
            rc = fp32(c) ? launch_step<3, float>(c, adapt, k) : launch_step<3, double>(c, adapt, k);
        if (rc) return rc;
    }
    c->wc_pending += nsteps;
    return PFG_OK;
}

int wc_sync(pfg_ctx* c, pfg_step_status* st) {
    std::memset(st, 0, sizeof(*st));
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, c->wc_dt.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    st->converged = 1;
    st->steps_done = c->wc_pending;
    st->dt = c->h_scalars[0];
    st->time = c->h_scalars[1];
    c->host_time = st->time;
    c->wc_pending = 0;
    return PFG_OK;
}

int wc_steps(pfg_ctx* c, double dt, int nsteps, pfg_step_status* st) {
    c->wc_pending = 0;
    int rc = wc_enqueue(c, dt, nsteps);
    if (rc) return rc;
    return wc_sync(c, st);
}

int wc_next_dt(pfg_ctx* c, double* dt) {
    const WcConst k = make_const(c);
    int rc;
    if (c->dim == 2)
        rc = fp32(c) ? dt_only<2, float>(c, k) : dt_only<2, double>(c, k);
    else
        rc = fp32(c) ? dt_only<3, float>(c, k) : dt_only<3, double>(c, k);
    if (rc) return rc;
    PFG_CUDA(c, cudaMemcpyAsync(dt, c->wc_dt.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_mass(pfg_ctx* c, double* out) {
    double* red = ptr<double>(c->red);
    double* res = red + c->max_grid * 4 + 40;
    unsigned* ticket = reinterpret_cast<unsigned*>(red + c->max_grid * 4 + 48);
    const GaussConst g = gauss_const(c->dim);
    const int grid = std::max(1, std::min(c->max_grid, div_up(std::max(c->E, 1), BLOCK)));
    if (c->dim == 2)
        k_wc_mass<2><<<grid, BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), c->ws.p,
                                                    fp32(c), g.refSize, red, ticket, res);
    else
        k_wc_mass<3><<<grid, BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), c->ws.p,
                                                    fp32(c), g.refSize, red, ticket, res);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, res, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    *out = c->h_scalars[0];
    return PFG_OK;
}

}  // namespace pfg
