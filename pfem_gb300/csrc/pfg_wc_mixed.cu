// Mixed-precision weakly compressible step: FP32 arithmetic only, double-float state.
//
// Same algorithm as pfg_wc.cu (SolverWCompNewton::m_solveWCompNewtonNoT, WCompNewton/
// Solver.cpp:236-276; ContEquation.inl:123-169,334-413; MomEquation.inl:201-374;
// computeNextDT Solver.cpp:192-234), arranged for GB300, whose FP64 pipe runs at 1/64 of the
// FP32 rate: a per-step kernel that issues FP64 instructions (even conversions) is bound by
// that pipe.  So nothing per step touches FP64:
//   * positions, velocities and pressures are double-float pairs (hi, lo: two FP32 numbers
//     whose sum carries ~48 significant bits), updated with error-free transforms (TwoSum);
//   * density is stored as rho - rho* (the deviation, ~1e-3 rho*) in FP32;
//   * element arithmetic is FP32; the two node-level cancellations are kept exact:
//       - Jacobian entries are differences of double-float coordinates (hi - hi is exact for
//         nearby nodes, Sterbenz), so geometry keeps ~1e-7 relative accuracy;
//       - pressure enters as differences p_j - p_i of double-float values;
//       - the p_i * sum_e A_fi term sums the (unscaled) adjugate entries as double-float, so
//         the patch sums that vanish at interior nodes stay ~1e-14 instead of FP32 noise.
// Only the device-side time accumulation (one thread) and the API conversions touch FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "pfg_device.cuh"
#include "pfg_fst.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

struct WcmConst {
    float K0, K0p, rho_star, mu, sc, max_dt;
    float kk;     // K0' / K0
    float ikp;    // 1 / K0'
    float g[3];
    int meduri;
    float MM[4][4];
    float s[4];
    float S;
    float refSize;
    float mu_sum;
};

WcmConst make_mconst(pfg_ctx* c) {
    const GaussConst gc = gauss_const(c->dim);
    WcmConst k{};
    k.K0 = (float)c->prm.K0;
    k.K0p = (float)c->prm.K0p;
    k.rho_star = (float)c->prm.rho_star;
    k.mu = (float)c->prm.mu;
    k.sc = (float)c->prm.security_coeff;
    k.max_dt = (float)c->prm.max_dt;
    k.kk = (float)(c->prm.K0p / c->prm.K0);
    k.ikp = (float)(1.0 / c->prm.K0p);
    for (int f = 0; f < 3; ++f) k.g[f] = (float)c->prm.gravity[f];
    k.meduri = c->prm.meduri;
    double S = 0, mus = 0;
    for (int i = 0; i < 4; ++i) {
        k.s[i] = (float)gc.s[i];
        if (i <= c->dim) S += gc.s[i];
        for (int j = 0; j < 4; ++j) k.MM[i][j] = (float)gc.MM[i][j];
    }
    for (int q = 0; q < gc.n; ++q) mus += c->prm.mu * gc.w[q];
    k.S = (float)S;
    k.refSize = (float)gc.refSize;
    k.mu_sum = (float)mus;
    return k;
}

// wc_dt: one 64-byte slot per instance (TSLOT doubles): doubles [dt, time, min, ticket], float dt
// at byte offset 32 and, for batched contexts, the running CFL minimum as FP32 bits at byte 36
enum : int { T_DT = 0, T_TIME = 1, T_MIN = 2, T_TICKET = 3 };
constexpr int TSLOT = 8;
constexpr unsigned MIN_NONE = 0x7f800000u;  // +inf: no candidate yet
__device__ __forceinline__ float* dtf_ptr(double* tdt) { return reinterpret_cast<float*>(tdt + 4); }
__device__ __forceinline__ unsigned* minbits_ptr(double* tdt) { return reinterpret_cast<unsigned*>(tdt + 4) + 1; }

// Independent meshes stored back to back in one context (pfg_set_instances on a mixed WC
// context): node -> instance map and per-instance [mu, mu sum_g w_g]; node_inst == nullptr
// for a single mesh.
struct WcInst {
    const int* node_inst;
    const float* f;
    __device__ __forceinline__ int of(int n) const { return node_inst ? __ldg(node_inst + n) : 0; }
};

// ---- error-free transforms ------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
// (hi, lo) += (xh, xl)
__device__ __forceinline__ void df_add(float& hi, float& lo, float xh, float xl) {
    float s, e;
    two_sum(hi, xh, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, xl));
    fast_two_sum(s, e, hi, lo);
}
// (ah, al) * (bh, bl)
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
    const float p = __fmul_rn(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    fast_two_sum(p, e, ph, pl);
}

// State layout (floats):
//   XH[d][N] XL[d][N] | VH0 VL0 VH1 VL1 [d][N] | PH0 PL0 PH1 PL1 [N] | RD[N] | AX[d][N]
// v and p have two halves; `cur` selects the current one (the step works in place on one).
struct St {
    float *xh, *xl, *vh, *vl, *ph, *pl, *rd, *ax;
};
__host__ __device__ inline St state_ptrs(float* base, int dim, int N, int cur) {
    St s;
    s.xh = base;
    s.xl = base + (size_t)dim * N;
    s.vh = base + (size_t)(2 + 2 * cur) * dim * N;
    s.vl = base + (size_t)(3 + 2 * cur) * dim * N;
    float* pb = base + (size_t)6 * dim * N;
    s.ph = pb + (size_t)2 * cur * N;
    s.pl = s.ph + N;
    s.rd = pb + (size_t)4 * N;
    s.ax = s.rd + N;
    return s;
}
inline size_t state_floats(int dim, int N) { return (size_t)(7 * dim + 5) * N; }

// Coordinate differences of double-float positions in FP32 (hi - hi is exact for nearby nodes).
struct PosDF {
    const float *xh, *xl;
    int N;
    __device__ __forceinline__ float operator()(int a, int b, int d) const {
        const size_t ia = (size_t)d * N + a, ib = (size_t)d * N + b;
        return (xh[ia] - xh[ib]) + (xl[ia] - xl[ib]);
    }
};

// Element -> node exchange, incidence-major: the contribution of element e to its local node i
// goes to record q = inc_slot[e*(dim+1)+i], the position of (e, i) in node-major incidence
// order, so each node reads one contiguous run of records.  Records are padded to whole float4s
// and written with vector stores:
//   continuity: [ML, CONT]                                                  (float2)
//   momentum:   [MLR, FS_f (dim), WH_f (dim), WL_f (dim), HE, pad]          (2 / 3 float4)
// (the continuity records are consumed before the momentum records are written).  HE is the
// element's CFL length 2 Rin, from which each node takes the minimum over its elements.
template <int DIM>
struct Rec {
    static constexpr int MLR = 0, FS = 1, WH = 1 + DIM, WL = 1 + 2 * DIM, HE = 1 + 3 * DIM;
    static constexpr int MOM = (HE + 1 + 3) / 4 * 4;   // floats per momentum record (8 / 12)
};

// Jacobian from double-float coordinates: Jh exact differences of hi parts, Jl of lo parts.
template <int DIM>
__device__ __forceinline__ void jac_df(const St& st, int N, const int (&nd)[DIM + 1], float (&Jh)[DIM][DIM],
                                       float (&Jl)[DIM][DIM]) {
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
        const float oh = st.xh[(size_t)r * N + nd[0]], ol = st.xl[(size_t)r * N + nd[0]];
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
            Jh[r][c] = __fsub_rn(st.xh[(size_t)r * N + nd[c + 1]], oh);
            Jl[r][c] = __fsub_rn(st.xl[(size_t)r * N + nd[c + 1]], ol);
        }
    }
}

// Adjugate of J as double-float (adj = detJ * invJ), and per node k the unscaled area
// gradient G[f][k] = adj-based: A_fk = refSize * G[f][k].
template <int DIM>
__device__ __forceinline__ void adj_df(const float (&Jh)[DIM][DIM], const float (&Jl)[DIM][DIM],
                                       float (&Gh)[DIM][DIM + 1], float (&Gl)[DIM][DIM + 1]) {
    if constexpr (DIM == 2) {
        // adj = [[J11, -J01], [-J10, J00]]; dN_{k+1}/dx_f = adj[k][f] / detJ
        Gh[0][1] = Jh[1][1];
        Gl[0][1] = Jl[1][1];
        Gh[1][1] = -Jh[0][1];
        Gl[1][1] = -Jl[0][1];
        Gh[0][2] = -Jh[1][0];
        Gl[0][2] = -Jl[1][0];
        Gh[1][2] = Jh[0][0];
        Gl[1][2] = Jl[0][0];
    } else {
        // cofactor(a,b) = J[r1][c1] J[r2][c2] - J[r1][c2] J[r2][c1]; adj[k][f] = cofactor of J(f,k)
        auto cof = [&](int r1, int c1, int r2, int c2, float& h, float& l) {
            float p1h, p1l, p2h, p2l;
            df_mul(Jh[r1][c1], Jl[r1][c1], Jh[r2][c2], Jl[r2][c2], p1h, p1l);
            df_mul(Jh[r1][c2], Jl[r1][c2], Jh[r2][c1], Jl[r2][c1], p2h, p2l);
            h = p1h;
            l = p1l;
            df_add(h, l, -p2h, -p2l);
        };
        // invJ rows (Element.cpp:108-133) times detJ
        float ah[3][3], al[3][3];
        cof(1, 1, 2, 2, ah[0][0], al[0][0]);
        cof(2, 1, 0, 2, ah[0][1], al[0][1]);
        cof(0, 1, 1, 2, ah[0][2], al[0][2]);
        cof(2, 0, 1, 2, ah[1][0], al[1][0]);
        cof(0, 0, 2, 2, ah[1][1], al[1][1]);
        cof(1, 0, 0, 2, ah[1][2], al[1][2]);
        cof(1, 0, 2, 1, ah[2][0], al[2][0]);
        cof(2, 0, 0, 1, ah[2][1], al[2][1]);
        cof(0, 0, 1, 1, ah[2][2], al[2][2]);
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                Gh[f][k + 1] = ah[k][f];
                Gl[f][k + 1] = al[k][f];
            }
    }
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        float h = -Gh[f][1], l = -Gl[f][1];
#pragma unroll
        for (int k = 2; k <= DIM; ++k) df_add(h, l, -Gh[f][k], -Gl[f][k]);
        Gh[f][0] = h;
        Gl[f][0] = l;
    }
}

// det J from the double-float adjugate and Jacobian: (adj J)_00 = sum_f adj[0][f] J[f][0], with
// adj[0][f] = G[f][1] (adj_df).  The FP32 determinant of the rounded Jacobian loses ~1e-6 of its
// value to cancellation on 3D elements; this keeps the element size, and so the lumped masses,
// at FP32 rounding.
template <int DIM>
__device__ __forceinline__ float det_adj(const float (&Jh)[DIM][DIM], const float (&Jl)[DIM][DIM],
                                         const float (&Gh)[DIM][DIM + 1], const float (&Gl)[DIM][DIM + 1]) {
    float h = 0.0f, l = 0.0f;
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        float ph, pl;
        df_mul(Gh[f][1], Gl[f][1], Jh[f][0], Jl[f][0], ph, pl);
        df_add(h, l, ph, pl);
    }
    return h + l;
}

// Half-step velocity and position update of one node (the start of
// m_solveWCompNewtonNoT, WCompNewton/Solver.cpp:249-254): v += dt/2 a; x += dt v unless fixed.
// Evaluated where the values are first needed (continuity element kernel, for each element's
// nodes) and stored by the continuity node kernel; both evaluate the same operations.
template <int DIM>
__device__ __forceinline__ void predict_node(const St& st, int N, int n, bool fixed, float dt, float (&xh)[DIM],
                                             float (&xl)[DIM], float (&vh)[DIM], float (&vl)[DIM]) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const size_t k = (size_t)d * N + n;
        vh[d] = st.vh[k];
        vl[d] = st.vl[k];
        df_add(vh[d], vl[d], 0.5f * dt * st.ax[k], 0.0f);
        xh[d] = st.xh[k];
        xl[d] = st.xl[k];
        if (!fixed) df_add(xh[d], xl[d], dt * vh[d], dt * vl[d]);
    }
}

// Element size and CFL length h_e = 2 Rin from the Jacobian (Element::getRin, Element.cpp:226-294)
template <int DIM>
__device__ __forceinline__ float cfl_length(const float (&J)[DIM][DIM], float size) {
    if constexpr (DIM == 2) {
        const float e01 = sqrtf(J[0][0] * J[0][0] + J[1][0] * J[1][0]);
        const float e02 = sqrtf(J[0][1] * J[0][1] + J[1][1] * J[1][1]);
        const float dx = J[0][1] - J[0][0], dy = J[1][1] - J[1][0];
        const float e12 = sqrtf(dx * dx + dy * dy);
        return 2.0f * (size / ((e01 + e12 + e02) * 0.5f));
    } else {  // face areas from edge cross products
        float u[4][3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            u[1][a] = J[a][0];
            u[2][a] = J[a][1];
            u[3][a] = J[a][2];
            u[0][a] = 0.0f;
        }
        auto nrm = [&](int a0, int a1, int a2) {
            const float ux = u[a1][0] - u[a0][0], uy = u[a1][1] - u[a0][1], uz = u[a1][2] - u[a0][2];
            const float wx = u[a2][0] - u[a0][0], wy = u[a2][1] - u[a0][1], wz = u[a2][2] - u[a0][2];
            const float cx = uy * wz - uz * wy, cy = uz * wx - ux * wz, cz = ux * wy - uy * wx;
            return sqrtf(cx * cx + cy * cy + cz * cz);
        };
        const float sum = nrm(0, 1, 2) + nrm(0, 3, 2) + nrm(0, 1, 3) + nrm(3, 1, 2);
        return 2.0f * (6.0f * size / sum);
    }
}

// Continuity element kernel (m_buildSystemdpdt, ContEquation.inl:353-413) on the predicted
// positions and velocities, computed here from the state of the previous step.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_m_cont_elem(int E, int N, const int* __restrict__ conn,
                                                       const uint8_t* __restrict__ flags, St st,
                                                       const double* __restrict__ tdt, WcmConst k,
                                                       const int* __restrict__ slot, float* __restrict__ cb,
                                                       WcInst wi) {
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    const float dt = *dtf_ptr(const_cast<double*>(tdt) + TSLOT * wi.of(nd[0]));
    float xh[NPE][DIM], xl[NPE][DIM], vh[NPE][DIM], vl[NPE][DIM];
#pragma unroll
    for (int j = 0; j < NPE; ++j) predict_node<DIM>(st, N, nd[j], flags[nd[j]] & F_FIXED, dt, xh[j], xl[j], vh[j], vl[j]);
    float Jh[DIM][DIM], Jl[DIM][DIM], J[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
            Jh[r][c] = __fsub_rn(xh[c + 1][r], xh[0][r]);
            Jl[r][c] = __fsub_rn(xl[c + 1][r], xl[0][r]);
            J[r][c] = Jh[r][c] + Jl[r][c];
        }
    float Gh[DIM][NPE], Gl[DIM][NPE];
    adj_df<DIM>(Jh, Jl, Gh, Gl);
    const float ae = det_adj<DIM>(Jh, Jl, Gh, Gl) * k.refSize;
    float ph[NPE], pl[NPE];
    float adiv = 0;
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        ph[j] = st.ph[nd[j]];
        pl[j] = st.pl[nd[j]];
#pragma unroll
        for (int f = 0; f < DIM; ++f) adiv += (Gh[f][j] + Gl[f][j]) * vh[j][f];
    }
    adiv *= k.refSize;  // |e| div v
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        const int q = __ldg(slot + (size_t)e * NPE + i);
        float mp = 0, mdp = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            mp += k.MM[i][j] * ph[j];
            mdp += k.MM[i][j] * ((ph[j] - ph[i]) + (pl[j] - pl[i]));
        }
        const float swn = k.K0 * k.s[i] + k.K0p * mp;
        float cont = -dt * swn * adiv;
        if (k.meduri) cont += ae * mdp;
        reinterpret_cast<float2*>(cb)[q] = make_float2(ae * k.s[i], cont);
    }
}

// Continuity node kernel: stores the node's predicted position and velocity, sums its
// continuity records (ContEquation.inl:396-409), applies the free-node BC and Tait EOS.
template <int DIM>
__global__ void k_m_cont_node(int N, const int* __restrict__ ne_ptr, const uint8_t* __restrict__ flags,
                              const float* __restrict__ cb, WcmConst k, St st, double* __restrict__ tdt,
                              WcInst wi) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (!wi.node_inst && n == 0) tdt[T_TIME] += (double)*dtf_ptr(tdt);  // Problem::updateTime
    if (n >= N) return;
    const float dt = *dtf_ptr(tdt + TSLOT * wi.of(n));
    const uint8_t fl = flags[n];
    {
        float xh[DIM], xl[DIM], vh[DIM], vl[DIM];
        predict_node<DIM>(st, N, n, fl & F_FIXED, dt, xh, xl, vh, vl);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const size_t kk = (size_t)d * N + n;
            st.vh[kk] = vh[d];
            st.vl[kk] = vl[d];
            st.xh[kk] = xh[d];
            st.xl[kk] = xl[d];
        }
    }
    float m = 0, f0 = 0;
    const float2* r2 = reinterpret_cast<const float2*>(cb);
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const float2 c2 = r2[q];
        m += c2.x;
        f0 += c2.y;
    }
    if (fl & F_FREE) {
        st.ph[n] = 0.0f;
        st.pl[n] = 0.0f;
        st.rd[n] = 0.0f;
        return;
    }
    float ph = st.ph[n], pl = st.pl[n];
    df_add(ph, pl, f0 / m, 0.0f);
    st.ph[n] = ph;
    st.pl[n] = pl;
    // rho - rho* = rho* expm1(log1p(K0' p / K0) / K0')
    st.rd[n] = k.rho_star * expm1f(log1pf(k.kk * ph) * k.ikp);
}

// Momentum element kernel (MomEquation.inl:229-302) and the element's CFL length.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_m_mom_elem(int E, int N, const int* __restrict__ conn, St st, WcmConst k,
                                                      const int* __restrict__ slot, float* __restrict__ cb,
                                                      WcInst wi) {
    using L = Rec<DIM>;
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    const float mu_sum = wi.f ? wi.f[2 * wi.of(nd[0]) + 1] : k.mu_sum;
    float Jh[DIM][DIM], Jl[DIM][DIM], J[DIM][DIM];
    jac_df<DIM>(st, N, nd, Jh, Jl);
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int c = 0; c < DIM; ++c) J[r][c] = Jh[r][c] + Jl[r][c];
    float Gh[DIM][NPE], Gl[DIM][NPE], A[DIM][NPE];
    adj_df<DIM>(Jh, Jl, Gh, Gl);
    const float det = det_adj<DIM>(Jh, Jl, Gh, Gl);
    const float ae = det * k.refSize;
    const float he = cfl_length<DIM>(J, ae);
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int j = 0; j < NPE; ++j) A[f][j] = k.refSize * (Gh[f][j] + Gl[f][j]);
    float V[DIM][NPE], Rh[NPE], ph[NPE], pl[NPE];
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        ph[j] = st.ph[nd[j]];
        pl[j] = st.pl[nd[j]];
        Rh[j] = k.rho_star + st.rd[nd[j]];
#pragma unroll
        for (int f = 0; f < DIM; ++f) V[f][j] = st.vh[(size_t)f * N + nd[j]];
    }
    float Lg[DIM][DIM];
    float divA = 0;
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int b = 0; b < DIM; ++b) {
            float t = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) t += A[b][j] * V[a][j];
            Lg[a][b] = t;
        }
#pragma unroll
    for (int a = 0; a < DIM; ++a) divA += Lg[a][a];
    const float kf = mu_sum / ae;
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        const int q = __ldg(slot + (size_t)e * NPE + i);
        float rec[L::MOM];
#pragma unroll
        for (int r = 0; r < L::MOM; ++r) rec[r] = 0.0f;
        float mr = 0, dp = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            mr += k.MM[i][j] * Rh[j];
            dp += k.s[j] * ((ph[j] - ph[i]) + (pl[j] - pl[i]));
        }
        const float mlr = ae * mr;
        rec[L::MLR] = mlr;
        float gg[NPE];
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            float t = 0;
#pragma unroll
            for (int f = 0; f < DIM; ++f) t += A[f][i] * A[f][j];
            gg[j] = t;
        }
#pragma unroll
        for (int f1 = 0; f1 < DIM; ++f1) {
            float kv = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) kv += gg[j] * V[f1][j];
#pragma unroll
            for (int f2 = 0; f2 < DIM; ++f2) kv += A[f2][i] * Lg[f2][f1];
            kv -= (2.0f / 3.0f) * A[f1][i] * divA;
            rec[L::FS + f1] = -kf * kv + A[f1][i] * dp + mlr * k.g[f1];
            rec[L::WH + f1] = Gh[f1][i];
            rec[L::WL + f1] = Gl[f1][i];
        }
        rec[L::HE] = he;
        float4* dst = reinterpret_cast<float4*>(cb + (size_t)q * L::MOM);
#pragma unroll
        for (int v = 0; v < L::MOM / 4; ++v) dst[v] = make_float4(rec[4 * v], rec[4 * v + 1], rec[4 * v + 2], rec[4 * v + 3]);
    }
}

// Momentum node kernel (MomEquation.inl:201-226,279-374): sums the node's records, adds the
// surface tension of its free-surface facets (in FP32), applies the BCs, updates acceleration
// and velocity.  With `cfl`, also the CFL time step of the next
// step (computeNextDT, WCompNewton/Solver.cpp:192-234): the reference's minimum over elements
// of sc^2 h_e^2 / max_{nodes of e} max(|u|^2, c^2, 4 alpha^2 / h_e^2) equals the minimum over
// nodes of the same expression at the node's smallest incident h_e (it grows with h_e), and in
// FP32 the two orders give the same bits (every operation is monotone).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_m_mom_node(int N, const int* __restrict__ ne_ptr,
                                                      const uint8_t* __restrict__ flags, const float* __restrict__ cb,
                                                      const double* __restrict__ vbc, double* __restrict__ tdt,
                                                      WcmConst k, St st, float* __restrict__ partials,
                                                      const float* __restrict__ fst, WcInst wi, bool cfl) {
    using L = Rec<DIM>;
    __shared__ float sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int inst = n < N ? wi.of(n) : 0;
    const float dt = *dtf_ptr(tdt + TSLOT * inst);
    float best = 3.0e38f;
    if (n < N) {
        float m = 0, F[DIM], Wh[DIM], Wl[DIM];
        float hmin = 3.0e38f;
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] = Wh[f] = Wl[f] = 0;
        const int q0 = ne_ptr[n], q1 = ne_ptr[n + 1];
        for (int q = q0; q < q1; ++q) {
            float rec[L::MOM];
            const float4* src = reinterpret_cast<const float4*>(cb + (size_t)q * L::MOM);
#pragma unroll
            for (int v = 0; v < L::MOM / 4; ++v) {
                const float4 t = src[v];
                rec[4 * v] = t.x;
                rec[4 * v + 1] = t.y;
                rec[4 * v + 2] = t.z;
                rec[4 * v + 3] = t.w;
            }
            m += rec[L::MLR];
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                F[f] += rec[L::FS + f];
                df_add(Wh[f], Wl[f], rec[L::WH + f], rec[L::WL + f]);
            }
            hmin = fminf(hmin, rec[L::HE]);
        }
        const float pS = st.ph[n] * k.S * k.refSize;
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] += pS * (Wh[f] + Wl[f]);
        if (fst)
#pragma unroll
            for (int f = 0; f < DIM; ++f) F[f] += fst[(size_t)f * N + n];
        float inv = 1.0f / m;
        const uint8_t fl = flags[n];
        if ((fl & F_FREE) && !(fl & F_BOUND)) {
#pragma unroll
            for (int f = 0; f < DIM; ++f) F[f] = k.g[f];
            inv = 1.0f;
        } else if ((fl & F_BOUND) && (fl & F_DIRICHLET)) {
            // Dirichlet values are host-provided FP64; read as float pairs written at set time
            const float* vb = reinterpret_cast<const float*>(vbc);
#pragma unroll
            for (int f = 0; f < DIM; ++f) F[f] = vb[(size_t)f * N + n];
            inv = 1.0f;
        }
        float u2 = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            const size_t kk = (size_t)f * N + n;
            const float a = inv * F[f];
            st.ax[kk] = a;
            float vh = st.vh[kk], vl = st.vl[kk];
            df_add(vh, vl, 0.5f * dt * a, 0.0f);
            st.vh[kk] = vh;
            st.vl[kk] = vl;
            u2 += vh * vh;
        }
        if (cfl && q1 > q0) {
            const float rho = k.rho_star + st.rd[n];
            const float m1 = fmaxf(u2, (k.K0 + k.K0p * st.ph[n]) / rho);
            const float m2 = (wi.f ? wi.f[2 * inst] : k.mu) / rho;
            const float maxSq = fmaxf(m1, 4.0f * m2 * m2 / (hmin * hmin));
            best = k.sc * k.sc * hmin * hmin / maxSq;
        }
    }
    if (!cfl) return;
    if (wi.node_inst) {
        // per-instance minimum: atomic min of the (positive) FP32 bit patterns, one atomic per
        // warp when the warp's nodes belong to one instance (min is exact in any order)
        const int i0 = __shfl_sync(0xffffffffu, inst, 0);
        if (__all_sync(0xffffffffu, n >= N || inst == i0)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_down_sync(0xffffffffu, best, o));
            if ((threadIdx.x & 31) == 0 && best < 3.0e38f)
                atomicMin(minbits_ptr(tdt + TSLOT * i0), __float_as_uint(best));
        } else if (n < N && best < 3.0e38f) {
            atomicMin(minbits_ptr(tdt + TSLOT * inst), __float_as_uint(best));
        }
        return;
    }
    // grid minimum: block minimum, then the last block to finish reduces the block minima
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_down_sync(0xffffffffu, best, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = best;
    __syncthreads();
    if (wid == 0) {
        best = lane < BLOCK / 32 ? sh[lane] : 3.0e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_down_sync(0xffffffffu, best, o));
    }
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
    float mn = 3.0e38f;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) mn = fminf(mn, __ldcg(partials + i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
    __syncthreads();
    if (lane == 0) sh[wid] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = 3.0e38f;
        for (int w = 0; w < BLOCK / 32; ++w) r = fminf(r, sh[w]);
        const float dtn = fminf(sqrtf(r), k.max_dt);
        *dtf_ptr(tdt) = dtn;
        tdt[T_DT] = (double)dtn;
        tdt[T_MIN] = (double)r;
        *ticket = 0u;
    }
}

// CFL time step of the current state, element by element (used once per state upload; the
// step computes it inside k_m_mom_node).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_m_dt(int E, int N, const int* __restrict__ conn, St st,
                                                const float* __restrict__ nodal, WcmConst k,
                                                float* __restrict__ partials, double* __restrict__ tdt, WcInst wi) {
    __shared__ float sh[32];
    float best = 3.0e38f;
    if (wi.node_inst) {  // batched: each element's candidate to its instance's minimum
        for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
            int nd[DIM + 1];
            load_nodes<DIM>(conn, E, e, nd);
            float Jh[DIM][DIM], Jl[DIM][DIM], J[DIM][DIM];
            jac_df<DIM>(st, N, nd, Jh, Jl);
#pragma unroll
            for (int r = 0; r < DIM; ++r)
#pragma unroll
                for (int c = 0; c < DIM; ++c) J[r][c] = Jh[r][c] + Jl[r][c];
            float Gh[DIM][DIM + 1], Gl[DIM][DIM + 1];
            adj_df<DIM>(Jh, Jl, Gh, Gl);
            const float he = cfl_length<DIM>(J, det_adj<DIM>(Jh, Jl, Gh, Gl) * k.refSize);
            float m1 = 0, m2 = 0;
#pragma unroll
            for (int a = 0; a <= DIM; ++a) {
                m1 = fmaxf(m1, nodal[nd[a]]);
                m2 = fmaxf(m2, nodal[(size_t)N + nd[a]]);
            }
            const float maxSq = fmaxf(m1, 4.0f * m2 * m2 / (he * he));
            atomicMin(minbits_ptr(tdt + TSLOT * wi.of(nd[0])), __float_as_uint(k.sc * k.sc * he * he / maxSq));
        }
        return;
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        int nd[DIM + 1];
        load_nodes<DIM>(conn, E, e, nd);
        float Jh[DIM][DIM], Jl[DIM][DIM], J[DIM][DIM];
        jac_df<DIM>(st, N, nd, Jh, Jl);
#pragma unroll
        for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int c = 0; c < DIM; ++c) J[r][c] = Jh[r][c] + Jl[r][c];
        float Gh[DIM][DIM + 1], Gl[DIM][DIM + 1];
        adj_df<DIM>(Jh, Jl, Gh, Gl);
        const float he = cfl_length<DIM>(J, det_adj<DIM>(Jh, Jl, Gh, Gl) * k.refSize);
        float m1 = 0, m2 = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) {
            m1 = fmaxf(m1, nodal[nd[a]]);
            m2 = fmaxf(m2, nodal[(size_t)N + nd[a]]);
        }
        const float maxSq = fmaxf(m1, 4.0f * m2 * m2 / (he * he));
        best = fminf(best, k.sc * k.sc * he * he / maxSq);
    }
    // block min
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_down_sync(0xffffffffu, best, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = best;
    __syncthreads();
    if (wid == 0) {
        best = lane < BLOCK / 32 ? sh[lane] : 3.0e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_down_sync(0xffffffffu, best, o));
    }
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
    float mn = 3.0e38f;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) mn = fminf(mn, ((volatile float*)partials)[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
    __syncthreads();
    if (lane == 0) sh[wid] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = 3.0e38f;
        for (int w = 0; w < BLOCK / 32; ++w) r = fminf(r, sh[w]);
        const float dt = fminf(sqrtf(r), k.max_dt);
        *dtf_ptr(tdt) = dt;
        tdt[T_DT] = (double)dt;
        tdt[T_MIN] = (double)r;
        *ticket = 0u;
    }
}

template <int DIM>
__global__ void k_m_nodal(int N, St st, WcmConst k, float* __restrict__ nodal, WcInst wi) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float u2 = 0;
#pragma unroll
    for (int f = 0; f < DIM; ++f) u2 += st.vh[(size_t)f * N + n] * st.vh[(size_t)f * N + n];
    const float rho = k.rho_star + st.rd[n];
    nodal[n] = fmaxf(u2, (k.K0 + k.K0p * st.ph[n]) / rho);
    nodal[(size_t)N + n] = (wi.f ? wi.f[2 * wi.of(n)] : k.mu) / rho;
}

// Batched contexts, after a step (advance = 1) or a CFL evaluation: each instance's slot takes
// its new time step dt = min(sqrt(min), maxDT) from the collected minimum (adaptive mode), the
// time advances by the step's dt (Problem::updateTime), and the minimum is reset.
__global__ void k_m_finalize(int n_inst, double* __restrict__ tdt, float max_dt, int adapt, int advance) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_inst) return;
    double* t = tdt + TSLOT * i;
    if (advance) t[T_TIME] += (double)*dtf_ptr(t);
    unsigned* mb = minbits_ptr(t);
    if (adapt && *mb != MIN_NONE) {
        const float r = __uint_as_float(*mb);
        const float dtn = fminf(sqrtf(r), max_dt);
        *dtf_ptr(t) = dtn;
        t[T_DT] = (double)dtn;
        t[T_MIN] = (double)r;
    }
    *mb = MIN_NONE;
}

// ---- API conversions (FP64, outside the step) -------------------------------------------
__device__ __forceinline__ void split(double x, float& h, float& l) {
    h = (float)x;
    l = (float)(x - (double)h);
}

__global__ void k_m_from_double(int N, int dim, const double* __restrict__ s, const double* __restrict__ pos,
                                double rho_star, St st) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    for (int d = 0; d < dim; ++d) {
        const size_t k = (size_t)d * N + n;
        if (s) {
            split(s[k], st.vh[k], st.vl[k]);
            st.ax[k] = (float)s[(size_t)(dim + 2 + d) * N + n];
        }
        if (pos) split(pos[k], st.xh[k], st.xl[k]);
    }
    if (s) {
        split(s[(size_t)dim * N + n], st.ph[n], st.pl[n]);
        st.rd[n] = (float)(s[(size_t)(dim + 1) * N + n] - rho_star);
    }
}

__global__ void k_m_to_double(int N, int dim, St st, double rho_star, double* __restrict__ s,
                              double* __restrict__ pos) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    for (int d = 0; d < dim; ++d) {
        const size_t k = (size_t)d * N + n;
        if (s) {
            s[k] = (double)st.vh[k] + (double)st.vl[k];
            s[(size_t)(dim + 2 + d) * N + n] = (double)st.ax[k];
        }
        if (pos) pos[k] = (double)st.xh[k] + (double)st.xl[k];
    }
    if (s) {
        s[(size_t)dim * N + n] = (double)st.ph[n] + (double)st.pl[n];
        s[(size_t)(dim + 1) * N + n] = rho_star + (double)st.rd[n];
    }
}

__global__ void k_m_vbc(int n, const double* __restrict__ vbc, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)vbc[i];
}

St st_of(pfg_ctx* c) { return state_ptrs(ptr<float>(c->ws), c->dim, c->N, c->wc_cur); }

WcInst wi_of(pfg_ctx* c) {
    return c->n_wc_inst > 1 ? WcInst{ptr<int>(c->node_inst), ptr<float>(c->wc_inst)} : WcInst{nullptr, nullptr};
}

template <int DIM>
int launch_mstep(pfg_ctx* c, bool adapt, const WcmConst& k) {
    const int N = c->N, E = c->E;
    St st = st_of(c);
    float* cb = ptr<float>(c->wc_el);
    const int* slot = ptr<int>(c->inc_slot);
    // block minima of the CFL reduction go to the per-node CFL scratch (unused during a step)
    float* partials = ptr<float>(c->wc_nodal);
    double* tdt = ptr<double>(c->wc_dt);
    const double* vbcf = reinterpret_cast<const double*>(ptr<float>(c->wc_eld));  // FP32 Dirichlet values
    const int gn = div_up(N, BLOCK), ge = std::max(1, div_up(E, BLOCK));
    const uint8_t* flags = ptr<uint8_t>(c->flags);
    const WcInst wi = wi_of(c);
    if (E > 0) {
        prof_begin(c, PH_WC_CONT_ELEM);
        k_m_cont_elem<DIM><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), flags, st, tdt, k, slot, cb, wi);
        prof_end(c, PH_WC_CONT_ELEM);
    }
    prof_begin(c, PH_WC_CONT_NODE);
    k_m_cont_node<DIM><<<gn, BLOCK, 0, c->stream>>>(N, ptr<int>(c->ne_ptr), flags, cb, k, st, tdt, wi);
    prof_end(c, PH_WC_CONT_NODE);
    if (E > 0) {
        prof_begin(c, PH_WC_MOM_ELEM);
        k_m_mom_elem<DIM><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), st, k, slot, cb, wi);
        prof_end(c, PH_WC_MOM_ELEM);
    }
    prof_begin(c, PH_WC_MOM_NODE);
    const FstArgs fa = fst_args(c);
    if (fa.nodes)
        k_fst<DIM, float><<<div_up(fa.n_nodes, BLOCK), BLOCK, 0, c->stream>>>(
            fa, E, ptr<int>(c->conn), PosDF{st.xh, st.xl, N}, N, ptr<float>(c->fst_force));
    k_m_mom_node<DIM><<<gn, BLOCK, 0, c->stream>>>(N, ptr<int>(c->ne_ptr), flags, cb, vbcf, tdt, k, st, partials,
                                                   fst_force<float>(c), wi, adapt && E > 0);
    if (wi.node_inst)  // batched: each instance's new dt and time
        k_m_finalize<<<div_up(c->n_wc_inst, 128), 128, 0, c->stream>>>(c->n_wc_inst, tdt, k.max_dt, adapt && E > 0, 1);
    prof_end(c, PH_WC_MOM_NODE);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

}  // namespace

size_t wcm_state_bytes(pfg_ctx* c) { return sizeof(float) * state_floats(c->dim, c->N); }

size_t wcm_elem_bytes(pfg_ctx* c) {
    const int rec = c->dim == 2 ? Rec<2>::MOM : Rec<3>::MOM;
    return sizeof(float) * (size_t)rec * (c->dim + 1) * std::max(c->E, 1);
}

int wcm_launch_step(pfg_ctx* c, bool adapt) {
    const WcmConst k = make_mconst(c);
    return c->dim == 2 ? launch_mstep<2>(c, adapt, k) : launch_mstep<3>(c, adapt, k);
}

// positions: c->pos (double) -> double-float state (after upload)
int wcm_positions_in(pfg_ctx* c) {
    k_m_from_double<<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, c->dim, nullptr, ptr<double>(c->pos),
                                                                  c->prm.rho_star, st_of(c));
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

// double-float positions -> c->pos (before any FP64 consumer reads them)
int wcm_positions_out(pfg_ctx* c) {
    k_m_to_double<<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, c->dim, st_of(c), c->prm.rho_star, nullptr,
                                                                ptr<double>(c->pos));
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

int wcm_set_states(pfg_ctx* c, const double* h) {
    const size_t n = (size_t)(2 * c->dim + 2) * c->N;
    int rc = ensure(c, c->stage, sizeof(double) * n);
    if (rc) return rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->stage.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    k_m_from_double<<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, c->dim, ptr<double>(c->stage), nullptr,
                                                                  c->prm.rho_star, st_of(c));
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wcm_get_states(pfg_ctx* c, double* h) {
    const size_t n = (size_t)(2 * c->dim + 2) * c->N;
    int rc = ensure(c, c->stage, sizeof(double) * n);
    if (rc) return rc;
    k_m_to_double<<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, c->dim, st_of(c), c->prm.rho_star,
                                                                ptr<double>(c->stage), nullptr);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaMemcpyAsync(h, c->stage.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

// FP64 image of the state in ctx->stage (device), for FP64 reductions
int wcm_state_to_stage(pfg_ctx* c) {
    k_m_to_double<<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, c->dim, st_of(c), c->prm.rho_star,
                                                                ptr<double>(c->stage), nullptr);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

// FP32 copy of the Dirichlet velocities (kept in wc_eld, unused by the mixed step otherwise)
int wcm_vbc_refresh(pfg_ctx* c) {
    const int n = c->dim * c->N;
    k_m_vbc<<<div_up(n, BLOCK), BLOCK, 0, c->stream>>>(n, ptr<double>(c->vbc), ptr<float>(c->wc_eld));
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

int wcm_next_dt(pfg_ctx* c) {
    const WcmConst k = make_mconst(c);
    const int N = c->N, E = c->E;
    if (E == 0) return fail(c, PFG_ERR_STATE, "no elements");
    St st = st_of(c);
    float* nodal = ptr<float>(c->wc_nodal);
    const int grid = std::min(c->max_grid, div_up(E, BLOCK));
    float* partials = reinterpret_cast<float*>(ptr<double>(c->red));
    const WcInst wi = wi_of(c);
    if (c->dim == 2) {
        k_m_nodal<2><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, st, k, nodal, wi);
        k_m_dt<2><<<grid, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), st, nodal, k, partials, ptr<double>(c->wc_dt),
                                                 wi);
    } else {
        k_m_nodal<3><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, st, k, nodal, wi);
        k_m_dt<3><<<grid, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), st, nodal, k, partials, ptr<double>(c->wc_dt),
                                                 wi);
    }
    if (wi.node_inst)
        k_m_finalize<<<div_up(c->n_wc_inst, 128), 128, 0, c->stream>>>(c->n_wc_inst, ptr<double>(c->wc_dt), k.max_dt,
                                                                      1, 0);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

// Independent meshes stored back to back (node_off), each with its own viscosity; every
// instance gets its own time-step slot, initialised from the context's current one.
__global__ void k_m_slots_init(int n_inst, double* __restrict__ tdt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_inst) return;
    double* t = tdt + TSLOT * i;
    if (i > 0)
        for (int k = 0; k < TSLOT; ++k) t[k] = tdt[k];
    *minbits_ptr(t) = MIN_NONE;
}

int wcm_set_instances(pfg_ctx* c, int n_inst, const int* node_off, const double* mu) {
    wc_release_graphs(c);
    const GaussConst gc = gauss_const(c->dim);
    std::vector<float> f((size_t)2 * n_inst);
    std::vector<int> node_inst((size_t)std::max(c->N, 1));
    for (int i = 0; i < n_inst; ++i) {
        double mus = 0;
        for (int q = 0; q < gc.n; ++q) mus += mu[i] * gc.w[q];
        f[2 * i] = (float)mu[i];
        f[2 * i + 1] = (float)mus;
        for (int n = node_off[i]; n < node_off[i + 1]; ++n) node_inst[n] = i;
    }
    int rc;
    // the first slot keeps its contents: copy it out before the buffer may move
    double slot0[TSLOT];
    PFG_CUDA(c, cudaMemcpyAsync(slot0, c->wc_dt.p, sizeof(slot0), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    if ((rc = ensure(c, c->wc_inst, sizeof(float) * f.size())) ||
        (rc = ensure(c, c->node_inst, sizeof(int) * node_inst.size())) ||
        (rc = ensure(c, c->wc_dt, sizeof(double) * TSLOT * (size_t)n_inst)))
        return rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->wc_dt.p, slot0, sizeof(slot0), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->wc_inst.p, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->node_inst.p, node_inst.data(), sizeof(int) * node_inst.size(),
                                cudaMemcpyHostToDevice, c->stream));
    k_m_slots_init<<<div_up(n_inst, 128), 128, 0, c->stream>>>(n_inst, ptr<double>(c->wc_dt));
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->n_wc_inst = n_inst;
    return PFG_OK;
}

}  // namespace pfg
