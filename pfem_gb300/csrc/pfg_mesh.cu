// Device-side topology of an uploaded mesh: node->element incidence, node adjacency, the
// node-pair list and the CSR sparsity pattern of the PSPG system.
//
// Pattern rule (derived from m_buildAbPSPG, MomContEquationPSPG.inl:55-128, and Eigen's
// setFromTriplets, :136): row r = n + f*N holds
//   * one diagonal entry when node n is free (in no element), or when n is bound and f < dim
//     (identity rows pushed at :108-128, element rows skipped at :68);
//   * otherwise columns m + f2*N for every node m sharing an element with n (n included) and
//     every field f2 = 0..dim, in ascending column order (field-major blocks, nodes ascending).
// The default (0,0,0.0) triplets of skipped slots (:17) only add 0.0 to entry (0,0), which the
// rule above always contains.  Row layout: position of column (m, f2) in row (n, f) is
//   row_ptr[r] + f2*deg(n) + rank of m in nbr(n).
#include <cuda_runtime.h>

#include <algorithm>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_CHUNK = BLOCK * SCAN_ITEMS;

// Exclusive scan of one chunk of `count` virtual items (item i = in[i] for i < n, else 0).
__global__ void k_scan_block(const int* __restrict__ in, int n, int count, int* __restrict__ out,
                             int* __restrict__ bsum) {
    __shared__ int sh[BLOCK];
    const long long base = (long long)blockIdx.x * SCAN_CHUNK;
    int v[SCAN_ITEMS];
    int tsum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        long long i = base + threadIdx.x * SCAN_ITEMS + k;
        v[k] = (i < n) ? in[i] : 0;
        tsum += v[k];
    }
    sh[threadIdx.x] = tsum;
    __syncthreads();
    for (int o = 1; o < BLOCK; o <<= 1) {
        int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - tsum;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        long long i = base + threadIdx.x * SCAN_ITEMS + k;
        if (i < count) out[i] = run;
        run += v[k];
    }
    if (threadIdx.x == BLOCK - 1 && bsum) bsum[blockIdx.x] = sh[BLOCK - 1];
}

__global__ void k_scan_add(int* __restrict__ out, int count, const int* __restrict__ boff) {
    const long long base = (long long)blockIdx.x * SCAN_CHUNK;
    const int add = boff[blockIdx.x];
    for (int k = threadIdx.x; k < SCAN_CHUNK; k += BLOCK) {
        long long i = base + k;
        if (i < count) out[i] += add;
    }
}

__global__ void k_count_incidence(const int* __restrict__ conn, int E, int npe, int* __restrict__ cnt) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)E * npe) return;
    atomicAdd(&cnt[conn[t]], 1);
}

__global__ void k_fill_incidence(const int* __restrict__ conn, int E, int npe, const int* __restrict__ ne_ptr,
                                 int* __restrict__ fill, int* __restrict__ ne_elem, uint8_t* __restrict__ ne_loc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)E * npe) return;
    const int k = (int)(t / E), e = (int)(t % E);
    const int n = conn[t];
    const int slot = atomicAdd(&fill[n], 1);
    ne_elem[ne_ptr[n] + slot] = e;
    ne_loc[ne_ptr[n] + slot] = (uint8_t)k;
}

// Sort each node's incident elements ascending (insertion sort; valence is small) and set the
// FREE flag of nodes in no element.
__global__ void k_sort_incidence(int N, const int* __restrict__ ne_ptr, int* __restrict__ ne_elem,
                                 uint8_t* __restrict__ ne_loc, uint8_t* __restrict__ flags) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int b = ne_ptr[n], eend = ne_ptr[n + 1];
    for (int i = b + 1; i < eend; ++i) {
        int e = ne_elem[i];
        uint8_t l = ne_loc[i];
        int j = i - 1;
        while (j >= b && ne_elem[j] > e) {
            ne_elem[j + 1] = ne_elem[j];
            ne_loc[j + 1] = ne_loc[j];
            --j;
        }
        ne_elem[j + 1] = e;
        ne_loc[j + 1] = l;
    }
    uint8_t f = flags[n] & (uint8_t)~F_FREE;
    if (eend == b) f |= F_FREE;
    flags[n] = f;
}

// Inverse of the sorted incidence lists: slot[e*npe + i] = position q of (e, i) in ne_elem,
// so an element kernel can write its contribution for local node i straight into the node's
// contiguous segment.
__global__ void k_incidence_slots(long long inc, int npe, const int* __restrict__ ne_elem,
                                  const uint8_t* __restrict__ ne_loc, int* __restrict__ slot) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= inc) return;
    slot[(size_t)ne_elem[q] * npe + ne_loc[q]] = (int)q;
}

// Sorted, de-duplicated neighbour list of node n (n included) in `list`; returns its size or
// -1 on overflow of MAX_NBR.
__device__ int gather_neighbours(int n, int npe, int E, const int* __restrict__ conn, const int* __restrict__ ne_ptr,
                                 const int* __restrict__ ne_elem, int* list) {
    int cnt = 1;
    list[0] = n;
    for (int k = ne_ptr[n]; k < ne_ptr[n + 1]; ++k) {
        const int e = ne_elem[k];
        for (int j = 0; j < npe; ++j) {
            const int m = conn[(size_t)j * E + e];
            int pos = 0;
            while (pos < cnt && list[pos] < m) ++pos;
            if (pos < cnt && list[pos] == m) continue;
            if (cnt == MAX_NBR) return -1;
            for (int q = cnt; q > pos; --q) list[q] = list[q - 1];
            list[pos] = m;
            ++cnt;
        }
    }
    return cnt;
}

__global__ void k_count_nbr(int N, int npe, int E, const int* __restrict__ conn, const int* __restrict__ ne_ptr,
                            const int* __restrict__ ne_elem, int* __restrict__ deg, int* __restrict__ err) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    int list[MAX_NBR];
    int c = gather_neighbours(n, npe, E, conn, ne_ptr, ne_elem, list);
    if (c < 0) {
        atomicOr(err, ERR_NBR_OVERFLOW);
        c = 1;
    }
    deg[n] = c;
}

__global__ void k_fill_nbr(int N, int npe, int E, const int* __restrict__ conn, const int* __restrict__ ne_ptr,
                           const int* __restrict__ ne_elem, const int* __restrict__ nbr_ptr, int* __restrict__ nbr,
                           int* __restrict__ pair_node) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    int list[MAX_NBR];
    int c = gather_neighbours(n, npe, E, conn, ne_ptr, ne_elem, list);
    const int b = nbr_ptr[n];
    const int cap = nbr_ptr[n + 1] - b;
    if (c < 0 || c > cap) c = cap;
    for (int i = 0; i < c; ++i) {
        nbr[b + i] = list[i];
        pair_node[b + i] = n;
    }
}

// Position of m in n's sorted neighbour list nbr[b0, b1) (m must be there).
__device__ __forceinline__ int nbr_rank(const int* __restrict__ nbr, int b0, int b1, int m) {
    int lo = b0, hi = b1 - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (nbr[mid] < m) lo = mid + 1;
        else hi = mid;
    }
    return lo - b0;
}

// Slots of the element-major element data of the mixed assembly: the elements in the order of
// their smallest node (ties by element index), so the elements that a run of consecutive nodes
// touches sit in a compact range of slots and the node and pair kernels' gathers hit L2.
// FILL = false counts, per node, the elements whose smallest node it is; FILL = true numbers
// them from the node's scanned base in its ascending incidence order.
// An element whose node list repeats its smallest node is numbered once, at the first of
// those local positions.
template <bool FILL>
__global__ void k_elem_slots(int N, int npe, int E, const int* __restrict__ conn, const int* __restrict__ ne_ptr,
                             const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                             int* __restrict__ count, const int* __restrict__ base, int* __restrict__ el_slot) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    int k = FILL ? base[n] : 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        int mn = conn[e], jm = 0;
        for (int j = 1; j < npe; ++j) {
            const int v = conn[(size_t)j * E + e];
            if (v < mn) {
                mn = v;
                jm = j;
            }
        }
        if (mn != n || ne_loc[q] != jm) continue;
        if (FILL) el_slot[e] = k;
        ++k;
    }
    if (!FILL) count[n] = k;
}

__global__ void k_ne_slots(long long inc, const int* __restrict__ ne_elem, const int* __restrict__ el_slot,
                           int* __restrict__ ne_slot) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < inc) ne_slot[q] = el_slot[ne_elem[q]];
}

// The connectivity in slot order (conn_s[k E + slot(e)] = conn[k E + e]): the element kernels
// that run over slots read it coalesced.
__global__ void k_conn_slots(int E, int npe, const int* __restrict__ conn, const int* __restrict__ el_slot,
                             int* __restrict__ conn_s) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int s = el_slot[e];
    for (int k = 0; k < npe; ++k) conn_s[(size_t)k * E + s] = conn[(size_t)k * E + e];
}

// Element lists of the off-diagonal node pairs: pair p = (n, m), m != n, lists every element
// containing both, ascending, as slot(e) * 16 + (local index of n) * 4 + (local index of m), and
// the same items with the element's position in n's incidence list instead of its slot (pe_pos,
// for the row-staged assembly).  One
// thread per node n owns the lists of n's pairs and walks n's sorted incidences, so each list
// comes out in ascending element order.  FILL = false counts, FILL = true writes.
template <bool FILL>
__global__ void k_pair_items(int N, int npe, int E, const int* __restrict__ conn, const int* __restrict__ ne_ptr,
                             const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                             const int* __restrict__ nbr_ptr, const int* __restrict__ nbr, int* __restrict__ cnt,
                             const int* __restrict__ pe_ptr, int* __restrict__ pe_item, int* __restrict__ pe_pair,
                             const int* __restrict__ el_slot, int* __restrict__ pe_pos) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int b0 = nbr_ptr[n], b1 = nbr_ptr[n + 1];
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        const int i = ne_loc[q];
        for (int j = 0; j < npe; ++j) {
            if (j == i) continue;
            const int p = b0 + nbr_rank(nbr, b0, b1, conn[(size_t)j * E + e]);
            if (FILL)
            {
                pe_pair[pe_ptr[p] + cnt[p]] = p;
                pe_pos[pe_ptr[p] + cnt[p]] = ((q - ne_ptr[n]) << 4) | (i << 2) | j;
                pe_item[pe_ptr[p] + cnt[p]++] = (el_slot[e] << 4) | (i << 2) | j;
            }
            else
                ++cnt[p];
        }
    }
}

__global__ void k_row_len(int N, int dim, const uint8_t* __restrict__ flags, const int* __restrict__ nbr_ptr,
                          int* __restrict__ len) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long R = (long long)(dim + 1) * N;
    if (r >= R) return;
    const int n = (int)(r % N), f = (int)(r / N);
    const uint8_t fl = flags[n];
    const bool single = (fl & F_FREE) || ((fl & F_BOUND) && f < dim);
    len[r] = single ? 1 : (nbr_ptr[n + 1] - nbr_ptr[n]) * (dim + 1);
}

__global__ void k_fill_cols(int N, int dim, const uint8_t* __restrict__ flags, const int* __restrict__ nbr_ptr,
                            const int* __restrict__ nbr, const int* __restrict__ row_ptr, int* __restrict__ col,
                            int* __restrict__ diag_pos) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long R = (long long)(dim + 1) * N;
    if (r >= R) return;
    const int n = (int)(r % N), f = (int)(r / N);
    const uint8_t fl = flags[n];
    const int rp = row_ptr[r];
    if ((fl & F_FREE) || ((fl & F_BOUND) && f < dim)) {
        col[rp] = (int)r;
        diag_pos[r] = rp;
        return;
    }
    const int b = nbr_ptr[n], deg = nbr_ptr[n + 1] - b;
    int self = 0;
    for (int k = 0; k < deg; ++k)
        if (nbr[b + k] == n) self = k;
    for (int f2 = 0; f2 <= dim; ++f2)
        for (int k = 0; k < deg; ++k) col[rp + f2 * deg + k] = nbr[b + k] + f2 * N;
    diag_pos[r] = rp + f * deg + self;
}

}  // namespace

int scan_exclusive(pfg_ctx* c, const int* in, int* out, int n, DBuf& tmp) {
    // level sizes
    std::vector<int> counts;
    int count = n + 1;
    size_t need = 0;
    while (true) {
        counts.push_back(count);
        int nb = div_up(count, SCAN_CHUNK);
        if (nb == 1) break;
        need += (size_t)nb + 1;
        count = nb;
    }
    int rc = ensure(c, tmp, std::max<size_t>(need, 1) * sizeof(int));
    if (rc) return rc;
    int* t = ptr<int>(tmp);
    // forward pass: level 0 scans `in` into `out`; level l scans block sums of level l-1
    std::vector<int*> lvl_out(counts.size());
    std::vector<int*> lvl_bsum(counts.size(), nullptr);
    size_t off = 0;
    for (size_t l = 0; l < counts.size(); ++l) {
        lvl_out[l] = (l == 0) ? out : lvl_bsum[l - 1];
        int nb = div_up(counts[l], SCAN_CHUNK);
        if (nb > 1) {
            lvl_bsum[l] = t + off;
            off += (size_t)nb + 1;
        }
    }
    for (size_t l = 0; l < counts.size(); ++l) {
        const int cnt = counts[l];
        const int nb = div_up(cnt, SCAN_CHUNK);
        const int* src = (l == 0) ? in : lvl_bsum[l - 1];
        const int nsrc = (l == 0) ? n : counts[l];
        // level l>0 scans its input in place into a copy: scan block sums of previous level
        if (l == 0) {
            k_scan_block<<<nb, BLOCK, 0, c->stream>>>(src, nsrc, cnt, lvl_out[l], lvl_bsum[l]);
        } else {
            k_scan_block<<<nb, BLOCK, 0, c->stream>>>(src, nsrc, cnt, lvl_bsum[l - 1], lvl_bsum[l]);
        }
        PFG_CHECK_LAUNCH(c);
    }
    for (int l = (int)counts.size() - 2; l >= 0; --l) {
        const int cnt = counts[l];
        const int nb = div_up(cnt, SCAN_CHUNK);
        int* dst = (l == 0) ? out : lvl_bsum[l - 1];
        k_scan_add<<<nb, BLOCK, 0, c->stream>>>(dst, cnt, lvl_bsum[l]);
        PFG_CHECK_LAUNCH(c);
    }
    return PFG_OK;
}

int build_topology(pfg_ctx* c) {
    const int N = c->N, E = c->E, npe = c->npe, dim = c->dim;
    DBuf tmp, cnt, fill, deg;
    int rc = 0;
    auto cleanup = [&]() {
        release(tmp);
        release(cnt);
        release(fill);
        release(deg);
    };
#define TRY(x)                \
    do {                      \
        rc = (x);             \
        if (rc) {             \
            cleanup();        \
            return rc;        \
        }                     \
    } while (0)
    const long long inc = (long long)E * npe;
    TRY(ensure(c, cnt, sizeof(int) * (size_t)N));
    TRY(ensure(c, fill, sizeof(int) * (size_t)N));
    TRY(ensure(c, c->ne_ptr, sizeof(int) * ((size_t)N + 1)));
    TRY(ensure(c, c->ne_elem, sizeof(int) * std::max<long long>(inc, 1)));
    TRY(ensure(c, c->ne_loc, std::max<long long>(inc, 1)));
    PFG_CUDA(c, cudaMemsetAsync(cnt.p, 0, sizeof(int) * N, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(fill.p, 0, sizeof(int) * N, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->err_word.p, 0, sizeof(int), c->stream));
    if (inc > 0) {
        k_count_incidence<<<div_up(inc, BLOCK), BLOCK, 0, c->stream>>>(ptr<int>(c->conn), E, npe, ptr<int>(cnt));
        PFG_CHECK_LAUNCH(c);
    }
    TRY(scan_exclusive(c, ptr<int>(cnt), ptr<int>(c->ne_ptr), N, tmp));
    if (inc > 0) {
        k_fill_incidence<<<div_up(inc, BLOCK), BLOCK, 0, c->stream>>>(ptr<int>(c->conn), E, npe, ptr<int>(c->ne_ptr),
                                                                        ptr<int>(fill), ptr<int>(c->ne_elem),
                                                                        ptr<uint8_t>(c->ne_loc));
        PFG_CHECK_LAUNCH(c);
    }
    k_sort_incidence<<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem),
                                                                ptr<uint8_t>(c->ne_loc), ptr<uint8_t>(c->flags));
    PFG_CHECK_LAUNCH(c);
    TRY(ensure(c, c->inc_slot, sizeof(int) * std::max<long long>(inc, 1)));
    if (inc > 0) {
        k_incidence_slots<<<div_up(inc, BLOCK), BLOCK, 0, c->stream>>>(inc, npe, ptr<int>(c->ne_elem),
                                                                       ptr<uint8_t>(c->ne_loc), ptr<int>(c->inc_slot));
        PFG_CHECK_LAUNCH(c);
    }

    // adjacency
    TRY(ensure(c, deg, sizeof(int) * (size_t)N));
    TRY(ensure(c, c->nbr_ptr, sizeof(int) * ((size_t)N + 1)));
    k_count_nbr<<<div_up(N, 128), 128, 0, c->stream>>>(N, npe, E, ptr<int>(c->conn), ptr<int>(c->ne_ptr),
                                                       ptr<int>(c->ne_elem), ptr<int>(deg), ptr<int>(c->err_word));
    PFG_CHECK_LAUNCH(c);
    TRY(scan_exclusive(c, ptr<int>(deg), ptr<int>(c->nbr_ptr), N, tmp));
    int hv[2];
    PFG_CUDA(c, cudaMemcpyAsync(&hv[0], ptr<int>(c->nbr_ptr) + N, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(&hv[1], c->err_word.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (hv[1] & ERR_NBR_OVERFLOW) {
        cleanup();
        return fail(c, PFG_ERR_DEVICE, "a node has more than %d neighbours", MAX_NBR);
    }
    c->P = hv[0];
    TRY(ensure(c, c->nbr, sizeof(int) * (size_t)c->P));
    TRY(ensure(c, c->pair_node, sizeof(int) * (size_t)c->P));
    k_fill_nbr<<<div_up(N, 128), 128, 0, c->stream>>>(N, npe, E, ptr<int>(c->conn), ptr<int>(c->ne_ptr),
                                                      ptr<int>(c->ne_elem), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr),
                                                      ptr<int>(c->pair_node));
    PFG_CHECK_LAUNCH(c);

    if (c->prm.kind == PFG_KIND_INCOMP_PSPG && c->prm.precision == PFG_PREC_MIXED) {
        // element lists of the off-diagonal node pairs (the FP32 pair assembly)
        if (E >= (1 << 27)) {
            cleanup();
            return fail(c, PFG_ERR_UNSUPPORTED, "too many elements for the pair element lists");
        }
        TRY(ensure(c, c->el_slot, sizeof(int) * (size_t)std::max(E, 1)));
        TRY(ensure(c, c->ne_slot, sizeof(int) * std::max<long long>(inc, 1)));
        k_elem_slots<false><<<div_up(N, 128), 128, 0, c->stream>>>(N, npe, E, ptr<int>(c->conn), ptr<int>(c->ne_ptr),
                                                                   ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc),
                                                                   ptr<int>(cnt), nullptr, nullptr);
        PFG_CHECK_LAUNCH(c);
        TRY(scan_exclusive(c, ptr<int>(cnt), ptr<int>(fill), N, tmp));
        k_elem_slots<true><<<div_up(N, 128), 128, 0, c->stream>>>(N, npe, E, ptr<int>(c->conn), ptr<int>(c->ne_ptr),
                                                                  ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc),
                                                                  nullptr, ptr<int>(fill), ptr<int>(c->el_slot));
        PFG_CHECK_LAUNCH(c);
        if (inc > 0) {
            k_ne_slots<<<div_up(inc, BLOCK), BLOCK, 0, c->stream>>>(inc, ptr<int>(c->ne_elem), ptr<int>(c->el_slot),
                                                                    ptr<int>(c->ne_slot));
            PFG_CHECK_LAUNCH(c);
        }
        TRY(ensure(c, c->conn_s, sizeof(int) * (size_t)npe * std::max(E, 1)));
        if (E > 0) {
            k_conn_slots<<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(E, npe, ptr<int>(c->conn), ptr<int>(c->el_slot),
                                                                    ptr<int>(c->conn_s));
            PFG_CHECK_LAUNCH(c);
        }
        TRY(ensure(c, cnt, sizeof(int) * (size_t)std::max(c->P, 1)));
        TRY(ensure(c, c->pe_ptr, sizeof(int) * ((size_t)c->P + 1)));
        PFG_CUDA(c, cudaMemsetAsync(cnt.p, 0, sizeof(int) * (size_t)c->P, c->stream));
        k_pair_items<false><<<div_up(N, 128), 128, 0, c->stream>>>(N, npe, E, ptr<int>(c->conn), ptr<int>(c->ne_ptr),
                                                                   ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc),
                                                                   ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<int>(cnt),
                                                                   nullptr, nullptr, nullptr, nullptr, nullptr);
        PFG_CHECK_LAUNCH(c);
        TRY(scan_exclusive(c, ptr<int>(cnt), ptr<int>(c->pe_ptr), c->P, tmp));
        const long long items = (long long)E * npe * (npe - 1);
        TRY(ensure(c, c->pe_item, sizeof(int) * (size_t)std::max<long long>(items, 1)));
        TRY(ensure(c, c->pe_pair, sizeof(int) * (size_t)std::max<long long>(items, 1)));
        TRY(ensure(c, c->pe_pos, sizeof(int) * (size_t)std::max<long long>(items, 1)));
        c->n_items = items;
        PFG_CUDA(c, cudaMemsetAsync(cnt.p, 0, sizeof(int) * (size_t)c->P, c->stream));
        k_pair_items<true><<<div_up(N, 128), 128, 0, c->stream>>>(N, npe, E, ptr<int>(c->conn), ptr<int>(c->ne_ptr),
                                                                  ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc),
                                                                  ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<int>(cnt),
                                                                  ptr<int>(c->pe_ptr), ptr<int>(c->pe_item),
                                                                  ptr<int>(c->pe_pair),
                                                                  ptr<int>(c->el_slot), ptr<int>(c->pe_pos));
        PFG_CHECK_LAUNCH(c);
    }

    if (c->prm.kind == PFG_KIND_INCOMP_PSPG) {
        const long long R = (long long)(dim + 1) * N;
        if (R > 0x7fffffffLL) {
            cleanup();
            return fail(c, PFG_ERR_UNSUPPORTED, "too many unknowns");
        }
        TRY(ensure(c, deg, sizeof(int) * (size_t)R));
        TRY(ensure(c, c->row_ptr, sizeof(int) * ((size_t)R + 1)));
        TRY(ensure(c, c->diag_pos, sizeof(int) * (size_t)R));
        k_row_len<<<div_up(R, BLOCK), BLOCK, 0, c->stream>>>(N, dim, ptr<uint8_t>(c->flags), ptr<int>(c->nbr_ptr),
                                                             ptr<int>(deg));
        PFG_CHECK_LAUNCH(c);
        TRY(scan_exclusive(c, ptr<int>(deg), ptr<int>(c->row_ptr), (int)R, tmp));
        int nnz = 0;
        PFG_CUDA(c, cudaMemcpyAsync(&nnz, ptr<int>(c->row_ptr) + R, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        c->nnz = nnz;
        TRY(ensure(c, c->col, sizeof(int) * (size_t)std::max(nnz, 1)));
        k_fill_cols<<<div_up(R, BLOCK), BLOCK, 0, c->stream>>>(N, dim, ptr<uint8_t>(c->flags), ptr<int>(c->nbr_ptr),
                                                               ptr<int>(c->nbr), ptr<int>(c->row_ptr), ptr<int>(c->col),
                                                               ptr<int>(c->diag_pos));
        PFG_CHECK_LAUNCH(c);
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    cleanup();
#undef TRY
    return PFG_OK;
}

}  // namespace pfg
