// Sparse LU of the PSPG system on the device: the plain form's direct solver
// (PFG_LINSOLVE_LU), standing where the reference factorises with Eigen's SparseLU after a
// COLAMD ordering, every Picard iteration (MomContEquationPSPG.inl:281-291,
// MomContEquation.hpp:6-12).
//
// Method (multifrontal, node blocks):
//   * ordering, once per mesh (host): nested dissection of the node graph by recursive
//     coordinate bisection - each step splits a node set at the median of its longest
//     coordinate axis and takes as separator the nodes of the lower half adjacent to the
//     upper half; sets of at most LU_LEAF nodes are leaves.  A fill-reducing ordering like
//     COLAMD's, but one whose elimination tree is balanced, so that the fronts of one tree
//     level factorise in parallel.  All d+1 unknowns of a node are eliminated together.
//   * symbolic analysis (host): for each tree node t ("front") its own nodes V_t (eliminated
//     there) and its boundary B_t (later nodes coupled to t's subtree), the list of matrix
//     blocks assembled into it and the map of its boundary into its parent's front.
//   * numeric factorisation (device), tree level by tree level from the leaves: each front is
//     a dense n_t x n_t FP64 matrix (n_t = (|V_t| + |B_t|)(d+1)) assembled from A and the
//     children's Schur complements, then partially factorised: its first m_t = |V_t|(d+1)
//     columns are eliminated with row pivoting among its m_t fully summed rows, leaving L, U
//     and the Schur complement of the boundary for the parent.  Small fronts: one thread block
//     each; large fronts: a blocked right-looking LU (panel, triangular solve, GEMM update).
//   * solve: forward substitution up the tree (each front's boundary contribution is added
//     into its parent's right-hand side, children in order: deterministic), backward
//     substitution down the tree, then FP64 iterative refinement against the CSR matrix (row
//     pivoting restricted to a front's fully summed rows is weaker than SparseLU's threshold
//     pivoting; refinement restores the direct solver's accuracy).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

constexpr int LU_LEAF = 48;          // nodes of a leaf front
constexpr int LU_SMALL = 192;        // fronts with n_t up to this factorise in one thread block
constexpr int LU_THREADS = 512;
constexpr int LU_NB = 32;            // panel width of the blocked factorisation
constexpr int LU_REFINE = 3;         // iterative-refinement sweeps after the direct solve

// ---- symbolic analysis (host) -----------------------------------------------------------------

struct Builder {
    int N, dim;
    const std::vector<int>& ptr;
    const std::vector<int>& nbr;
    const std::vector<double>& pos;  // dim x N
    std::vector<int> stamp;
    int stamp_id = 0;
    // tree
    std::vector<std::vector<int>> V;  // own nodes of each front
    std::vector<std::vector<int>> kids;
    std::vector<int> order;           // elimination order of the nodes
    std::vector<int> post;            // fronts in post-order

    Builder(int N_, int dim_, const std::vector<int>& p, const std::vector<int>& n, const std::vector<double>& x)
        : N(N_), dim(dim_), ptr(p), nbr(n), pos(x), stamp(N_, 0) {}

    int make(std::vector<int>& nodes) {
        const int id = (int)V.size();
        V.emplace_back();
        kids.emplace_back();
        if ((int)nodes.size() <= LU_LEAF) {
            V[id] = nodes;
            return id;
        }
        // longest axis of the bounding box, split at the median
        int axis = 0;
        double best = -1;
        for (int d = 0; d < dim; ++d) {
            double lo = 1e300, hi = -1e300;
            for (int v : nodes) {
                lo = std::min(lo, pos[(size_t)d * N + v]);
                hi = std::max(hi, pos[(size_t)d * N + v]);
            }
            if (hi - lo > best) {
                best = hi - lo;
                axis = d;
            }
        }
        const size_t half = nodes.size() / 2;
        std::nth_element(nodes.begin(), nodes.begin() + half, nodes.end(), [&](int a, int b) {
            const double xa = pos[(size_t)axis * N + a], xb = pos[(size_t)axis * N + b];
            return xa < xb || (xa == xb && a < b);
        });
        std::vector<int> L(nodes.begin(), nodes.begin() + half), R(nodes.begin() + half, nodes.end());
        ++stamp_id;
        for (int v : R) stamp[v] = stamp_id;
        std::vector<int> S, L2;
        for (int v : L) {
            bool sep = false;
            for (int k = ptr[v]; k < ptr[v + 1] && !sep; ++k) sep = stamp[nbr[k]] == stamp_id;
            (sep ? S : L2).push_back(v);
        }
        std::sort(S.begin(), S.end());
        V[id] = S;
        const int a = make(L2);
        const int b = make(R);
        kids[id] = {a, b};
        return id;
    }

    void postorder(int root) {
        // iterative post-order: children (in order) before the parent
        std::vector<std::pair<int, int>> st{{root, 0}};
        while (!st.empty()) {
            auto& [t, k] = st.back();
            if (k < (int)kids[t].size()) {
                const int c = kids[t][k++];
                st.push_back({c, 0});
            } else {
                post.push_back(t);
                for (int v : V[t]) order.push_back(v);
                st.pop_back();
            }
        }
    }
};

}  // namespace

namespace {

int lu_symbolic(pfg_ctx* c) {
    const int N = c->N, dim = c->dim, B = dim + 1;
    std::vector<int> ptr(N + 1), nbr(c->P);
    std::vector<double> pos((size_t)dim * N);
    PFG_CUDA(c, cudaMemcpyAsync(ptr.data(), c->nbr_ptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(nbr.data(), c->nbr.p, sizeof(int) * c->P, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(pos.data(), c->pos.p, sizeof(double) * pos.size(), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    Builder b(N, dim, ptr, nbr, pos);
    std::vector<int> all(N);
    std::iota(all.begin(), all.end(), 0);
    const int root = b.make(all);
    b.postorder(root);
    const int T = (int)b.V.size();
    std::vector<int> where(N);  // elimination position of each node
    for (int i = 0; i < N; ++i) where[b.order[i]] = i;
    std::vector<int> parent(T, -1), level(T, 0), last(T, -1);
    for (int t = 0; t < T; ++t)
        for (int k : b.kids[t]) parent[k] = t;
    for (int t : b.post) last[t] = b.V[t].empty() ? -1 : where[b.V[t].back()];
    // a front's last elimination position covers its subtree (post-order)
    for (int t : b.post) {
        for (int k : b.kids[t]) last[t] = std::max(last[t], last[k]);
    }
    for (int i = (int)b.post.size() - 1; i >= 0; --i) {
        const int t = b.post[i];
        if (parent[t] >= 0) level[t] = level[parent[t]] + 1;
    }
    // boundaries, bottom-up
    std::vector<std::vector<int>> Bn(T);
    std::vector<int> mark(N, -1);
    for (int t : b.post) {
        std::vector<int>& out = Bn[t];
        auto add = [&](int u) {
            if (where[u] > last[t] && mark[u] != t) {
                mark[u] = t;
                out.push_back(u);
            }
        };
        for (int v : b.V[t])
            for (int k = ptr[v]; k < ptr[v + 1]; ++k) add(nbr[k]);
        for (int k : b.kids[t])
            for (int u : Bn[k]) add(u);
        std::sort(out.begin(), out.end(), [&](int x, int y) { return where[x] < where[y]; });
    }
    // layout
    std::vector<LuFront> F(T);
    std::vector<int> nodes, recs, children, maps;
    long long mat = 0, vec = 0;
    int piv = 0;
    std::vector<int> local(N, -1);
    for (int t : b.post) {
        LuFront& f = F[t];
        f.nv = (int)b.V[t].size();
        f.nb = (int)Bn[t].size();
        f.node_off = (int)nodes.size();
        for (int v : b.V[t]) nodes.push_back(v);
        for (int u : Bn[t]) nodes.push_back(u);
        const int n = (f.nv + f.nb) * B;
        f.mat_off = mat;
        mat += (long long)n * n;
        f.vec_off = vec;
        vec += n;
        f.piv_off = piv;
        piv += f.nv * B;
        for (int k = 0; k < f.nv + f.nb; ++k) local[nodes[f.node_off + k]] = k;
        // assembly records: block (v, u) for v in V_t and u in V_t or B_t (from v's row), and
        // block (u, v) for u in B_t (from u's row): (local row, local col, row node, rank)
        f.rec_off = (int)(recs.size() / 4);
        const int first = f.nv ? where[b.V[t].front()] : 0;
        for (int v : b.V[t]) {
            for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
                const int u = nbr[k];
                if (where[u] < first) continue;  // eliminated in a descendant, assembled there
                recs.insert(recs.end(), {local[v], local[u], v, k - ptr[v]});
                if (local[u] >= f.nv) {
                    const int* ub = nbr.data() + ptr[u];
                    const int* ue = nbr.data() + ptr[u + 1];
                    const int rk = (int)(std::lower_bound(ub, ue, v) - ub);
                    recs.insert(recs.end(), {local[u], local[v], u, rk});
                }
            }
        }
        f.n_rec = (int)(recs.size() / 4) - f.rec_off;
        f.child_off = (int)children.size();
        f.n_child = (int)b.kids[t].size();
        for (int k : b.kids[t]) children.push_back(k);
        for (int k = 0; k < f.nv + f.nb; ++k) local[nodes[f.node_off + k]] = -1;
    }
    // boundary maps into the parent's front
    for (int t : b.post) {
        LuFront& f = F[t];
        f.map_off = (int)maps.size();
        const int p = parent[t];
        if (p < 0) continue;
        const LuFront& fp = F[p];
        for (int k = 0; k < fp.nv + fp.nb; ++k) local[nodes[fp.node_off + k]] = k;
        for (int k = 0; k < f.nb; ++k) maps.push_back(local[nodes[f.node_off + f.nv + k]]);
        for (int k = 0; k < fp.nv + fp.nb; ++k) local[nodes[fp.node_off + k]] = -1;
    }
    // every local index must address a row of its front (a bad one would write outside it)
    for (int t = 0; t < T; ++t) {
        const LuFront& f = F[t];
        const int nn = f.nv + f.nb;
        for (int q = f.rec_off; q < f.rec_off + f.n_rec; ++q)
            if (recs[4 * q] < 0 || recs[4 * q] >= nn || recs[4 * q + 1] < 0 || recs[4 * q + 1] >= nn)
                return fail(c, PFG_ERR_DEVICE, "LU analysis: assembly record outside front %d", t);
        if (parent[t] >= 0) {
            const LuFront& fp = F[parent[t]];
            for (int k = 0; k < f.nb; ++k) {
                const int li = maps[f.map_off + k];
                if (li < 0 || li >= fp.nv + fp.nb) return fail(c, PFG_ERR_DEVICE, "LU analysis: boundary map of front %d", t);
            }
        } else if (f.nb != 0) {
            return fail(c, PFG_ERR_DEVICE, "LU analysis: root front with a boundary");
        }
    }
    // level lists (deepest first), each split into small and large fronts
    int depth = 0;
    for (int t = 0; t < T; ++t) depth = std::max(depth, level[t]);
    c->lu_levels.assign(depth + 1, {});
    for (int t : b.post) c->lu_levels[depth - level[t]].push_back(t);
    // device copies
    const size_t need = sizeof(double) * (size_t)mat;
    int rc;
    if ((rc = ensure(c, c->lu_front, sizeof(LuFront) * T)) || (rc = ensure(c, c->lu_nodes, sizeof(int) * nodes.size())) ||
        (rc = ensure(c, c->lu_recs, sizeof(int) * std::max<size_t>(recs.size(), 4))) ||
        (rc = ensure(c, c->lu_kids, sizeof(int) * std::max<size_t>(children.size(), 1))) ||
        (rc = ensure(c, c->lu_maps, sizeof(int) * std::max<size_t>(maps.size(), 1))) ||
        (rc = ensure(c, c->lu_piv, sizeof(int) * std::max(piv, 1))) || (rc = ensure(c, c->lu_mat, need)) ||
        (rc = ensure(c, c->lu_vec, sizeof(double) * std::max<long long>(vec, 1))) ||
        (rc = ensure(c, c->lu_list, sizeof(int) * T)) || (rc = ensure(c, c->lu_r, sizeof(double) * c->R)))
        return rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->lu_front.p, F.data(), sizeof(LuFront) * T, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->lu_nodes.p, nodes.data(), sizeof(int) * nodes.size(), cudaMemcpyHostToDevice,
                                c->stream));
    if (!recs.empty())
        PFG_CUDA(c, cudaMemcpyAsync(c->lu_recs.p, recs.data(), sizeof(int) * recs.size(), cudaMemcpyHostToDevice,
                                    c->stream));
    if (!children.empty())
        PFG_CUDA(c, cudaMemcpyAsync(c->lu_kids.p, children.data(), sizeof(int) * children.size(),
                                    cudaMemcpyHostToDevice, c->stream));
    if (!maps.empty())
        PFG_CUDA(c, cudaMemcpyAsync(c->lu_maps.p, maps.data(), sizeof(int) * maps.size(), cudaMemcpyHostToDevice,
                                    c->stream));
    // level lists in one device array: small fronts of each level, then its large fronts
    std::vector<int> lists;
    c->lu_small.clear();
    c->lu_large.clear();
    for (auto& lv : c->lu_levels) {
        std::vector<int> sm, lg;
        for (int t : lv) ((F[t].nv + F[t].nb) * B <= LU_SMALL ? sm : lg).push_back(t);
        c->lu_small.push_back({(int)lists.size(), (int)sm.size()});
        lists.insert(lists.end(), sm.begin(), sm.end());
        c->lu_large.push_back(lg);
    }
    PFG_CUDA(c, cudaMemcpyAsync(c->lu_list.p, lists.data(), sizeof(int) * lists.size(), cudaMemcpyHostToDevice,
                                c->stream));
    c->h_lu_front.assign(F.begin(), F.end());
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->lu_fronts = T;
    c->lu_factor_bytes = need;
    c->lu_ready = true;
    return PFG_OK;
}

// ---- numeric factorisation (device) ------------------------------------------------------------

// Front t: zero, assemble its blocks of A (identity rows hold their diagonal), and add its
// children's Schur complements in child order.  One thread block per front.
template <int DIM>
__global__ void __launch_bounds__(LU_THREADS) k_lu_assemble(const int* __restrict__ list, const LuFront* __restrict__ F,
                                                            const int* __restrict__ recs, const int* __restrict__ kids,
                                                            const int* __restrict__ maps, int N,
                                                            const int* __restrict__ row_ptr,
                                                            const int* __restrict__ nbr_ptr,
                                                            const double* __restrict__ val, double* __restrict__ pool) {
    constexpr int B = DIM + 1;
    const LuFront f = F[list[blockIdx.x]];
    const int n = (f.nv + f.nb) * B;
    double* A = pool + f.mat_off;
    for (long long i = threadIdx.x; i < (long long)n * n; i += blockDim.x) A[i] = 0.0;
    __syncthreads();
    for (int r = threadIdx.x; r < f.n_rec * B * B; r += blockDim.x) {
        const int q = r / (B * B), f1 = (r / B) % B, f2 = r % B;
        const int* rc = recs + 4 * (size_t)(f.rec_off + q);
        const int lr = rc[0], lc = rc[1], v = rc[2], rank = rc[3];
        const int row = v + f1 * N;
        const int rp = row_ptr[row];
        double a;
        if (row_ptr[row + 1] - rp == 1)  // identity row: its diagonal only
            a = (f1 == f2 && lr == lc) ? val[rp] : 0.0;
        else
            a = val[rp + f2 * (nbr_ptr[v + 1] - nbr_ptr[v]) + rank];
        A[(size_t)(lr * B + f1) * n + lc * B + f2] = a;
    }
    __syncthreads();
    for (int k = 0; k < f.n_child; ++k) {
        const LuFront g = F[kids[f.child_off + k]];
        const int nc = (g.nv + g.nb) * B, mc = g.nv * B, sc = g.nb * B;
        const double* S = pool + g.mat_off;
        for (int r = threadIdx.x; r < sc * sc; r += blockDim.x) {
            const int i = r / sc, j = r % sc;
            const int li = maps[g.map_off + i / B] * B + i % B, lj = maps[g.map_off + j / B] * B + j % B;
            A[(size_t)li * n + lj] += S[(size_t)(mc + i) * nc + mc + j];
        }
        __syncthreads();
    }
}

// Pivot of column k among rows [k, m): the largest magnitude, ties to the lowest row.
__device__ __forceinline__ int lu_pivot(const double* A, int n, int k, int m, double* sv, int* si) {
    double best = -1.0;
    int bi = k;
    for (int i = k + threadIdx.x; i < m; i += blockDim.x) {
        const double a = fabs(A[(size_t)i * n + k]);
        if (a > best) {
            best = a;
            bi = i;
        }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            const double o = sv[threadIdx.x + s];
            const int oi = si[threadIdx.x + s];
            if (o > sv[threadIdx.x] || (o == sv[threadIdx.x] && oi < si[threadIdx.x])) {
                sv[threadIdx.x] = o;
                si[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    const int p = si[0];
    __syncthreads();
    return p;
}

// Column k of the elimination: pivot among rows [k, m), swap rows k and p over columns
// [0, n), scale column k below the diagonal, and update columns (k, c1) of rows (k, n).
__device__ __forceinline__ void lu_step(double* A, int n, int m, int k, int c1, int* piv, double* sv, int* si,
                                        int* err) {
    const int p = lu_pivot(A, n, k, m, sv, si);
    if (threadIdx.x == 0) {
        piv[k] = p;
        if (A[(size_t)p * n + k] == 0.0) atomicOr(err, 1);
    }
    if (p != k)
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const double t = A[(size_t)k * n + j];
            A[(size_t)k * n + j] = A[(size_t)p * n + j];
            A[(size_t)p * n + j] = t;
        }
    __syncthreads();
    const double d = A[(size_t)k * n + k];
    const double inv = d != 0.0 ? 1.0 / d : 0.0;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[(size_t)i * n + k] *= inv;
    __syncthreads();
    const int w = c1 - k - 1, h = n - k - 1;
    for (int r = threadIdx.x; r < h * w; r += blockDim.x) {
        const int i = k + 1 + r / w, j = k + 1 + r % w;
        A[(size_t)i * n + j] -= A[(size_t)i * n + k] * A[(size_t)k * n + j];
    }
    __syncthreads();
}

// Small fronts: the whole partial factorisation in one thread block.
__global__ void __launch_bounds__(LU_THREADS) k_lu_factor_small(const int* __restrict__ list,
                                                                const LuFront* __restrict__ F, int B,
                                                                double* __restrict__ pool, int* __restrict__ pivs,
                                                                int* __restrict__ err) {
    __shared__ double sv[LU_THREADS];
    __shared__ int si[LU_THREADS];
    const LuFront f = F[list[blockIdx.x]];
    const int n = (f.nv + f.nb) * B, m = f.nv * B;
    double* A = pool + f.mat_off;
    for (int k = 0; k < m; ++k) lu_step(A, n, m, k, n, pivs + f.piv_off, sv, si, err);
}

// Large fronts, blocked: panel [k0, k0 + kb) factorised (row swaps over all columns, updates
// inside the panel only) by one thread block ...
__global__ void __launch_bounds__(LU_THREADS) k_lu_panel(LuFront f, int B, int k0, int kb, double* __restrict__ pool,
                                                         int* __restrict__ pivs, int* __restrict__ err) {
    __shared__ double sv[LU_THREADS];
    __shared__ int si[LU_THREADS];
    const int n = (f.nv + f.nb) * B, m = f.nv * B;
    double* A = pool + f.mat_off;
    for (int k = k0; k < k0 + kb; ++k) lu_step(A, n, m, k, k0 + kb, pivs + f.piv_off, sv, si, err);
}

// ... the panel's rows of U to the right of it: U12 = L11^-1 A12 (unit lower L11), one
// thread per column ...
__global__ void k_lu_trsm(LuFront f, int B, int k0, int kb, double* __restrict__ pool) {
    const int n = (f.nv + f.nb) * B;
    const int j = k0 + kb + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double* A = pool + f.mat_off;
    for (int r = k0 + 1; r < k0 + kb; ++r) {
        double s = A[(size_t)r * n + j];
        for (int q = k0; q < r; ++q) s -= A[(size_t)r * n + q] * A[(size_t)q * n + j];
        A[(size_t)r * n + j] = s;
    }
}

// ... and the trailing update A22 -= L21 U12, 64 x 64 output tiles (4 x 4 per thread),
// operands staged in shared memory.
constexpr int GT = 64;
__global__ void __launch_bounds__(256) k_lu_gemm(LuFront f, int B, int k0, int kb, double* __restrict__ pool) {
    __shared__ double Ls[GT][LU_NB + 1];
    __shared__ double Us[LU_NB][GT + 1];
    const int n = (f.nv + f.nb) * B;
    const int s0 = k0 + kb;
    const int i0 = s0 + blockIdx.y * GT, j0 = s0 + blockIdx.x * GT;
    if (i0 >= n || j0 >= n) return;
    double* A = pool + f.mat_off;
    for (int r = threadIdx.x; r < GT * kb; r += blockDim.x) {
        const int i = r / kb, q = r % kb;
        Ls[i][q] = (i0 + i < n) ? A[(size_t)(i0 + i) * n + k0 + q] : 0.0;
    }
    for (int r = threadIdx.x; r < kb * GT; r += blockDim.x) {
        const int q = r / GT, j = r % GT;
        Us[q][j] = (j0 + j < n) ? A[(size_t)(k0 + q) * n + j0 + j] : 0.0;
    }
    __syncthreads();
    const int ti = (threadIdx.x / 16) * 4, tj = (threadIdx.x % 16) * 4;
    double acc[4][4] = {};
    for (int q = 0; q < kb; ++q) {
        double l[4], u[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            l[a] = Ls[ti + a][q];
            u[a] = Us[q][tj + a];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] += l[a] * u[b];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = i0 + ti + a, j = j0 + tj + b;
            if (i < n && j < n) A[(size_t)i * n + j] -= acc[a][b];
        }
}

// ---- solve ---------------------------------------------------------------------------------------

// Forward substitution of the fronts of a level: right-hand side of the own rows from b,
// boundary rows zero, plus the children's boundary contributions; row swaps; L y = P r over
// the fronts' columns; y and the boundary contribution w stay in the front's vector.
__global__ void __launch_bounds__(LU_THREADS) k_lu_forward(const int* __restrict__ list, int cnt,
                                                           const LuFront* __restrict__ F, int B, int N,
                                                           const int* __restrict__ nodes, const int* __restrict__ kids,
                                                           const int* __restrict__ maps, const double* __restrict__ pool,
                                                           const int* __restrict__ pivs, const double* __restrict__ b,
                                                           double* __restrict__ vec) {
    if ((int)blockIdx.x >= cnt) return;
    const LuFront f = F[list[blockIdx.x]];
    const int n = (f.nv + f.nb) * B, m = f.nv * B;
    const double* A = pool + f.mat_off;
    double* r = vec + f.vec_off;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int v = nodes[f.node_off + i / B];
        r[i] = i < m ? b[v + (size_t)(i % B) * N] : 0.0;
    }
    __syncthreads();
    for (int k = 0; k < f.n_child; ++k) {
        const LuFront g = F[kids[f.child_off + k]];
        const int mc = g.nv * B, sc = g.nb * B;
        const double* w = vec + g.vec_off + mc;
        for (int i = threadIdx.x; i < sc; i += blockDim.x) r[maps[g.map_off + i / B] * B + i % B] += w[i];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < m; ++k) {
            const int p = pivs[f.piv_off + k];
            if (p != k) {
                const double t = r[k];
                r[k] = r[p];
                r[p] = t;
            }
        }
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        const double yk = r[k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) r[i] -= A[(size_t)i * n + k] * yk;
        __syncthreads();
    }
}

// Backward substitution of the fronts of a level (parents before children): the boundary
// values from the solution, z = y - U12 x_B, U11 x_V = z, x_V to the solution.
__global__ void __launch_bounds__(LU_THREADS) k_lu_backward(const int* __restrict__ list, int cnt,
                                                            const LuFront* __restrict__ F, int B, int N,
                                                            const int* __restrict__ nodes,
                                                            const double* __restrict__ pool, double* __restrict__ vec,
                                                            double* __restrict__ x) {
    if ((int)blockIdx.x >= cnt) return;
    const LuFront f = F[list[blockIdx.x]];
    const int n = (f.nv + f.nb) * B, m = f.nv * B;
    const double* A = pool + f.mat_off;
    double* r = vec + f.vec_off;
    for (int i = m + threadIdx.x; i < n; i += blockDim.x) {
        const int u = nodes[f.node_off + i / B];
        r[i] = x[u + (size_t)(i % B) * N];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double s = r[i];
        for (int j = m; j < n; ++j) s -= A[(size_t)i * n + j] * r[j];
        r[i] = s;
    }
    __syncthreads();
    for (int k = m - 1; k >= 0; --k) {
        if (threadIdx.x == 0) r[k] /= A[(size_t)k * n + k];
        __syncthreads();
        const double xk = r[k];
        for (int i = threadIdx.x; i < k; i += blockDim.x) r[i] -= A[(size_t)i * n + k] * xk;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int v = nodes[f.node_off + i / B];
        x[v + (size_t)(i % B) * N] = r[i];
    }
}

// r = b - A x over the CSR rows (the refinement residual)
__global__ void k_lu_resid(int R, const int* __restrict__ rp, const int* __restrict__ col, const double* __restrict__ val,
                           const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R) return;
    double s = b[i];
    for (int k = rp[i]; k < rp[i + 1]; ++k) s -= val[k] * x[col[k]];
    r[i] = s;
}

__global__ void k_lu_add(int R, const double* __restrict__ d, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < R) x[i] += d[i];
}

template <int DIM>
int lu_factor(pfg_ctx* c) {
    constexpr int B = DIM + 1;
    const LuFront* F = ptr<LuFront>(c->lu_front);
    double* pool = ptr<double>(c->lu_mat);
    int* pivs = ptr<int>(c->lu_piv);
    int* err = ptr<int>(c->err_word);
    const int* list = ptr<int>(c->lu_list);
    for (size_t l = 0; l < c->lu_levels.size(); ++l) {
        const auto [off, cnt] = c->lu_small[l];
        const int nl = (int)c->lu_levels[l].size();
        // assemble every front of the level (small ones listed first in lu_levels' order too)
        if (cnt)
            k_lu_assemble<DIM><<<cnt, LU_THREADS, 0, c->stream>>>(list + off, F, ptr<int>(c->lu_recs), ptr<int>(c->lu_kids),
                                                                  ptr<int>(c->lu_maps), c->N, ptr<int>(c->row_ptr),
                                                                  ptr<int>(c->nbr_ptr), ptr<double>(c->val), pool);
        for (int t : c->lu_large[l]) {
            int* one = ptr<int>(c->lu_one) + t;
            k_lu_assemble<DIM><<<1, LU_THREADS, 0, c->stream>>>(one, F, ptr<int>(c->lu_recs), ptr<int>(c->lu_kids),
                                                                ptr<int>(c->lu_maps), c->N, ptr<int>(c->row_ptr),
                                                                ptr<int>(c->nbr_ptr), ptr<double>(c->val), pool);
        }
        if (cnt) k_lu_factor_small<<<cnt, LU_THREADS, 0, c->stream>>>(list + off, F, B, pool, pivs, err);
        for (int t : c->lu_large[l]) {
            const LuFront& f = c->h_lu_front[t];
            const int n = (f.nv + f.nb) * B, m = f.nv * B;
            for (int k0 = 0; k0 < m; k0 += LU_NB) {
                const int kb = std::min(LU_NB, m - k0);
                k_lu_panel<<<1, LU_THREADS, 0, c->stream>>>(f, B, k0, kb, pool, pivs, err);
                const int rest = n - k0 - kb;
                if (rest > 0) {
                    k_lu_trsm<<<div_up(rest, 128), 128, 0, c->stream>>>(f, B, k0, kb, pool);
                    const int tiles = div_up(rest, GT);
                    k_lu_gemm<<<dim3(tiles, tiles), 256, 0, c->stream>>>(f, B, k0, kb, pool);
                }
            }
        }
        (void)nl;
        PFG_CHECK_LAUNCH(c);
    }
    return PFG_OK;
}

int lu_solve_once(pfg_ctx* c, const double* b, double* x) {
    const int B = c->dim + 1;
    const LuFront* F = ptr<LuFront>(c->lu_front);
    const double* pool = ptr<double>(c->lu_mat);
    double* vec = ptr<double>(c->lu_vec);
    const int* list = ptr<int>(c->lu_list);
    const int* one = ptr<int>(c->lu_one);
    const int L = (int)c->lu_levels.size();
    for (int l = 0; l < L; ++l) {
        const auto [off, cnt] = c->lu_small[l];
        if (cnt)
            k_lu_forward<<<cnt, LU_THREADS, 0, c->stream>>>(list + off, cnt, F, B, c->N, ptr<int>(c->lu_nodes),
                                                            ptr<int>(c->lu_kids), ptr<int>(c->lu_maps), pool,
                                                            ptr<int>(c->lu_piv), b, vec);
        for (int t : c->lu_large[l])
            k_lu_forward<<<1, LU_THREADS, 0, c->stream>>>(one + t, 1, F, B, c->N, ptr<int>(c->lu_nodes),
                                                          ptr<int>(c->lu_kids), ptr<int>(c->lu_maps), pool,
                                                          ptr<int>(c->lu_piv), b, vec);
    }
    for (int l = L - 1; l >= 0; --l) {
        const auto [off, cnt] = c->lu_small[l];
        if (cnt)
            k_lu_backward<<<cnt, LU_THREADS, 0, c->stream>>>(list + off, cnt, F, B, c->N, ptr<int>(c->lu_nodes), pool,
                                                             vec, x);
        for (int t : c->lu_large[l])
            k_lu_backward<<<1, LU_THREADS, 0, c->stream>>>(one + t, 1, F, B, c->N, ptr<int>(c->lu_nodes), pool, vec, x);
    }
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

}  // namespace

void lu_release(pfg_ctx* c) {
    c->lu_ready = false;
    c->lu_levels.clear();
    c->lu_small.clear();
    c->lu_large.clear();
    c->h_lu_front.clear();
}

// A x = b with the current CSR system (b = the assembled right-hand side): factorise, solve,
// refine.  The factorisation's symbolic part is built once per mesh.
int lu_solve(pfg_ctx* c, double* x, int* refine_sweeps) {
    int rc;
    if (!c->lu_ready) {
        if ((rc = lu_symbolic(c))) return rc;
        std::vector<int> ids(c->lu_fronts);
        std::iota(ids.begin(), ids.end(), 0);
        if ((rc = ensure(c, c->lu_one, sizeof(int) * ids.size()))) return rc;
        PFG_CUDA(c, cudaMemcpyAsync(c->lu_one.p, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice,
                                    c->stream));
    }
    PFG_CUDA(c, cudaMemsetAsync(c->err_word.p, 0, sizeof(int), c->stream));
    if ((rc = c->dim == 2 ? lu_factor<2>(c) : lu_factor<3>(c))) return rc;
    const double* b = ptr<double>(c->rhs);
    if ((rc = lu_solve_once(c, b, x))) return rc;
    double* r = ptr<double>(c->lu_r);
    double* d = ptr<double>(c->kv);  // a Krylov vector as the correction
    const int R = c->R;
    for (int s = 0; s < LU_REFINE; ++s) {
        k_lu_resid<<<div_up(R, BLOCK), BLOCK, 0, c->stream>>>(R, ptr<int>(c->row_ptr), ptr<int>(c->col),
                                                              ptr<double>(c->val), b, x, r);
        PFG_CUDA(c, cudaMemsetAsync(d, 0, sizeof(double) * R, c->stream));
        if ((rc = lu_solve_once(c, r, d))) return rc;
        k_lu_add<<<div_up(R, BLOCK), BLOCK, 0, c->stream>>>(R, d, x);
        PFG_CHECK_LAUNCH(c);
    }
    *refine_sweeps = LU_REFINE;
    int h_err = 0;
    PFG_CUDA(c, cudaMemcpyAsync(&h_err, c->err_word.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (h_err & 1) return fail(c, PFG_ERR_DEVICE, "LU: zero pivot");
    return PFG_OK;
}

}  // namespace pfg
