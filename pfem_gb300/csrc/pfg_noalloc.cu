// CFL time step without any device allocation (pfg_wc_next_dt_noalloc).
//
// Same computation as pfg_next_dt on a plain (FP64) weakly compressible context: per-node
// max(u^2, c^2) and mu/rho, then per element sc^2 he^2 / max(...) reduced to the minimum and
// dt = min(sqrt(min), maxDT).  The difference is where the scratch lives.  pfg_next_dt keeps its
// per-node quantities and reduction partials in buffers the context allocated with cudaMalloc;
// this variant takes every input and the output from the caller and keeps its scratch in one
// file-scope device array, so a call performs no cudaMalloc, cudaFree or other allocation.
//
// Who needs this: code that is not allowed to allocate device memory at the point where it
// needs a time step.  Examples are a host application that hands all GPU memory to its own
// pool allocator up front and forbids cudaMalloc afterwards (cudaMalloc can synchronise the
// device and stall the application's other streams), a time loop running under someone
// else's stream capture, where an allocation call is illegal or breaks the capture, and
// plugins that only ever receive device pointers from their host.
//
// Limits and sharing rules:
//   * at most NOALLOC_MAX_NODES nodes; larger meshes are rejected with PFG_ERR_INVALID;
//   * the array lives on every device that loads the library until the process exits;
//   * all calls share the array and it keeps the last call's contents; the reduction counter is
//     cleared at the start of every call, the other scratch is fully overwritten before use;
//   * calls whose kernels overlap on the GPU (different streams, no ordering between them)
//     race on the shared array: order them on one stream or serialise them;
//   * the first call on each device looks up the array's device address (cudaGetSymbolAddress
//     with that device current); make that first call before any stream capture begins.  The
//     address is cached per device index for the life of the process: a cudaDeviceReset (or
//     any teardown of the device's primary context) between calls would leave it stale;
//   * connectivity indices are trusted: the caller guarantees 0 <= d_conn[k] < n_nodes;
//   * NaN: fmin/fmax drop a NaN operand, so an element with a NaN state is skipped and the
//     step stays finite, as std::min skips a NaN candidate in the reference's element loop
//     (WCompNewton/Solver.cpp:222; its NaN check at :230 therefore never sees one there).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace {

constexpr int NOALLOC_MAX_NODES = 1 << 20;
constexpr int NOALLOC_MAX_BLOCKS = 2048;
// layout: [nodal: 2*NOALLOC_MAX_NODES doubles][partials: NOALLOC_MAX_BLOCKS doubles][ticket]
constexpr size_t NOALLOC_DOUBLES = 2 * (size_t)NOALLOC_MAX_NODES + NOALLOC_MAX_BLOCKS + 32;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
double* g_scratch_addr[MAX_DEVICES] = {};

struct DtConst {
    double K0, K0p, mu, sc, max_dt, refSize;
};

template <int DIM>
__global__ void k_na_nodal(int N, const double* __restrict__ s, DtConst k, double* __restrict__ nodal) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double u2 = 0;
#pragma unroll
    for (int f = 0; f < DIM; ++f) u2 += s[(size_t)f * N + n] * s[(size_t)f * N + n];
    const double p = s[(size_t)DIM * N + n], rho = s[(size_t)(DIM + 1) * N + n];
    nodal[n] = fmax(u2, (k.K0 + k.K0p * p) / rho);
    nodal[(size_t)N + n] = k.mu / rho;
}

template <int DIM>
__global__ void __launch_bounds__(pfg::BLOCK) k_na_dt(int E, int N, const int* __restrict__ conn,
                                                      const double* __restrict__ pos, const double* __restrict__ nodal,
                                                      DtConst k, double* __restrict__ partials,
                                                      unsigned* __restrict__ ticket, double* __restrict__ out) {
    using namespace pfg;
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
        double he;
        if constexpr (DIM == 2) {  // Element::getRin 2D (Element.cpp:228-241)
            const double j00 = X[1][0] - X[0][0], j01 = X[2][0] - X[0][0];
            const double j10 = X[1][1] - X[0][1], j11 = X[2][1] - X[0][1];
            const double size = (j00 * j11 - j10 * j01) * k.refSize;
            auto dist = [&](int a, int b) {
                const double dx = X[a][0] - X[b][0], dy = X[a][1] - X[b][1];
                return sqrt(dx * dx + dy * dy);
            };
            const double sp = (dist(0, 1) + dist(1, 2) + dist(0, 2)) / 2;
            he = 2 * (size / sp);
        } else {  // Element::getRin 3D (Element.cpp:242-293)
            Geom<3> g;
            compute_geom<3>(pos, N, nd, g);
            const double size = g.detJ * k.refSize;
            auto nrm = [&](int a0, int a1, int a2) {
                const double ux = X[a1][0] - X[a0][0], uy = X[a1][1] - X[a0][1], uz = X[a1][2] - X[a0][2];
                const double wx = X[a2][0] - X[a0][0], wy = X[a2][1] - X[a0][1], wz = X[a2][2] - X[a0][2];
                const double cx = uy * wz - uz * wy, cy = uz * wx - ux * wz, cz = ux * wy - uy * wx;
                return sqrt(cx * cx + cy * cy + cz * cz);
            };
            const double sum = nrm(0, 1, 2) + nrm(0, 3, 2) + nrm(0, 1, 3) + nrm(3, 1, 2);
            he = 2 * (6 * size / sum);
        }
        double m1 = 0, m2 = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) {
            m1 = fmax(m1, nodal[nd[a]]);
            m2 = fmax(m2, nodal[(size_t)N + nd[a]]);
        }
        const double maxSq = fmax(m1, 4 * m2 * m2 / (he * he));
        best = fmin(best, k.sc * k.sc * he * he / maxSq);
    }
    best = block_min<BLOCK>(best, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = best;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double mn = 1.79769313486231570e308;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) mn = fmin(mn, ((volatile double*)partials)[i]);
    mn = block_min<BLOCK>(mn, sh);
    if (threadIdx.x == 0) {
        *out = fmin(sqrt(mn), k.max_dt);
        *ticket = 0u;
    }
}

// Device address of the scratch array on the current device (looked up once per device).
int scratch_address(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return PFG_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PFG_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return PFG_OK;
}

}  // namespace

extern "C" PFG_API int pfg_wc_next_dt_noalloc(const pfg_params* params, int32_t n_nodes, int32_t n_elems,
                                              const int32_t* d_conn, const double* d_pos, const double* d_states,
                                              double* d_dt, void* stream) {
    using namespace pfg;
    if (!params || !d_conn || !d_pos || !d_states || !d_dt) return PFG_ERR_INVALID;
    if (params->dim != 2 && params->dim != 3) return PFG_ERR_INVALID;
    if (n_nodes <= 0 || n_nodes > NOALLOC_MAX_NODES || n_elems <= 0) return PFG_ERR_INVALID;
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    double* nodal = scratch;
    double* partials = scratch + 2 * (size_t)NOALLOC_MAX_NODES;
    unsigned* ticket = reinterpret_cast<unsigned*>(partials + NOALLOC_MAX_BLOCKS);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the reduction counter must start at zero whatever the last call left behind
    if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), s) != cudaSuccess) return PFG_ERR_CUDA;
    const GaussConst g = gauss_const(params->dim);
    DtConst k{params->K0, params->K0p, params->mu, params->security_coeff, params->max_dt, g.refSize};
    const int gn = div_up(n_nodes, BLOCK);
    const int ge = std::max(1, std::min(NOALLOC_MAX_BLOCKS, div_up(n_elems, BLOCK)));
    if (params->dim == 2) {
        k_na_nodal<2><<<gn, BLOCK, 0, s>>>(n_nodes, d_states, k, nodal);
        k_na_dt<2><<<ge, BLOCK, 0, s>>>(n_elems, n_nodes, d_conn, d_pos, nodal, k, partials, ticket, d_dt);
    } else {
        k_na_nodal<3><<<gn, BLOCK, 0, s>>>(n_nodes, d_states, k, nodal);
        k_na_dt<3><<<ge, BLOCK, 0, s>>>(n_elems, n_nodes, d_conn, d_pos, nodal, k, partials, ticket, d_dt);
    }
    return cudaGetLastError() == cudaSuccess ? PFG_OK : PFG_ERR_CUDA;
}
