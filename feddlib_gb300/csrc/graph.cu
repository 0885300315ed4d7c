// graph.cu -- device construction of incidences, node adjacency and CSR
// patterns (built once per mesh).
//
// Replaces the pattern FEDDLib obtains from Tpetra: FE::addFeBlock /
// addFeBlockMatrix insert every dof pair of every node pair of an element
// (feddlib/core/FE/FE_def.hpp:1419-1442, 982-1062) and fillComplete sorts the
// columns and merges duplicates (Matrix_decl.hpp:133-138).  Here: per row
// node, the union of the column nodes of its incident elements, sorted and
// made unique by one warp (segmented bitonic sort in shared memory); the
// scalar CSR follows as node pattern x (dofs_r x dofs_c) blocks.
#include "engine.hpp"

namespace fedd {

namespace {

constexpr int kCand = 1024;  // candidate buffer per warp (>= kMaxIncidence * 10)
constexpr int kGraphWarps = 4;

__global__ void k_count_inc(const int32_t *__restrict__ conn, int npe, int64_t ne, int64_t nnodes,
                            int32_t *cnt, int *err) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ne * npe) return;
    int a = (int)(t / ne);
    int64_t e = t - (int64_t)a * ne;
    int32_t n = conn[(int64_t)a * ne + e];
    if (n < 0 || n >= nnodes) {
        set_dev_error(err, kDevMesh);
        return;
    }
    atomicAdd(&cnt[n], 1);
}

__global__ void k_fill_inc(const int32_t *__restrict__ conn, int npe, int64_t ne, int64_t nnodes,
                           const int64_t *__restrict__ ptr, int32_t *cursor, uint32_t *inc) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ne * npe) return;
    int a = (int)(t / ne);
    int64_t e = t - (int64_t)a * ne;
    int32_t n = conn[(int64_t)a * ne + e];
    if (n < 0 || n >= nnodes) return;
    int pos = atomicAdd(&cursor[n], 1);
    inc[ptr[n] + pos] = ((uint32_t)e << 4) | (uint32_t)a;
}

// the fill order above depends on atomic timing: sort each list so that the
// incidence order (and with it the summation order) is fixed: by the node's
// local index in the element, then by element, so that a row kernel meets the
// incidences sharing a local index (and its rows of the reference tables) in
// one run
__device__ __forceinline__ uint32_t inc_key(uint32_t v) { return ((v & 15u) << 28) | (v >> 4); }

__global__ void k_sort_inc(const int64_t *__restrict__ ptr, uint32_t *inc, int64_t nnodes, int *err,
                           int *maxinc) {
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nnodes) return;
    int64_t b = ptr[n], m = ptr[n + 1] - b;
    if (m > kMaxIncidence) {
        set_dev_error(err, kDevCapacity);
        return;
    }
    atomicMax(maxinc, (int)m);
    uint32_t v[kMaxIncidence];
    for (int i = 0; i < m; i++) v[i] = inc[b + i];
    for (int i = 1; i < m; i++) {
        uint32_t x = v[i];
        int j = i - 1;
        while (j >= 0 && inc_key(v[j]) > inc_key(x)) {
            v[j + 1] = v[j];
            j--;
        }
        v[j + 1] = x;
    }
    for (int i = 0; i < m; i++) inc[b + i] = v[i];
}

// warp-level bitonic sort of buf[0..np) (np a power of two >= 32)
__device__ void warp_bitonic(int32_t *buf, int np, int lane) {
    for (int k = 2; k <= np; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < np; i += 32) {
                int p = i ^ j;
                if (p > i) {
                    int32_t x = buf[i], y = buf[p];
                    bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        buf[i] = y;
                        buf[p] = x;
                    }
                }
            }
            __syncwarp();
        }
}

// gathers the column nodes of node n's incidences, sorts them and makes them
// unique into uniq[]; returns the number of unique nodes (or -1 on overflow)
__device__ int node_union(int64_t n, const int64_t *__restrict__ ptr, const uint32_t *__restrict__ inc,
                          const int32_t *__restrict__ col_conn, int npe_col, int64_t ne, int32_t *buf,
                          int32_t *uniq, int lane) {
    int64_t b = ptr[n];
    int m = (int)(ptr[n + 1] - b);
    int cnt = m * npe_col;
    if (cnt > kCand) return -1;
    int np = 32;
    while (np < cnt) np <<= 1;
    for (int i = lane; i < np; i += 32) {
        int32_t v = 0x7fffffff;
        if (i < cnt) {
            int k = i / npe_col, j = i - k * npe_col;
            uint32_t e = inc[b + k] >> 4;
            v = col_conn[(int64_t)j * ne + e];
        }
        buf[i] = v;
    }
    __syncwarp();
    warp_bitonic(buf, np, lane);
    int K = 0;
    for (int base = 0; base < cnt; base += 32) {
        int i = base + lane;
        bool f = i < cnt && (i == 0 || buf[i] != buf[i - 1]);
        unsigned bal = __ballot_sync(0xffffffffu, f);
        int pos = K + __popc(bal & ((1u << lane) - 1u));
        if (f && pos < kMaxAdjacency) uniq[pos] = buf[i];
        K += __popc(bal);
    }
    __syncwarp();
    return K;
}

__global__ void k_adj_count(const int64_t *__restrict__ ptr, const uint32_t *__restrict__ inc,
                            const int32_t *__restrict__ col_conn, int npe_col, int64_t ne, int64_t nnodes,
                            int64_t *cnt, int *err, int *maxadj) {
    __shared__ int32_t sbuf[kGraphWarps][kCand];
    __shared__ int32_t suni[kGraphWarps][kMaxAdjacency + 1];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t n = blockIdx.x * (int64_t)kGraphWarps + w;
    if (n >= nnodes) return;
    int K = node_union(n, ptr, inc, col_conn, npe_col, ne, sbuf[w], suni[w], lane);
    if (lane == 0) {
        if (K < 0 || K > kMaxAdjacency) {
            set_dev_error(err, kDevCapacity);
            K = 0;
        }
        cnt[n] = K;
        atomicMax(maxadj, K);
    }
}

__global__ void k_adj_fill(const int64_t *__restrict__ ptr, const uint32_t *__restrict__ inc,
                           const int32_t *__restrict__ col_conn, int npe_col, int64_t ne, int64_t nnodes,
                           const int64_t *__restrict__ adj_ptr, int32_t *adj, uint8_t *slots, int slot_off) {
    __shared__ int32_t sbuf[kGraphWarps][kCand];
    __shared__ int32_t suni[kGraphWarps][kMaxAdjacency + 1];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t n = blockIdx.x * (int64_t)kGraphWarps + w;
    if (n >= nnodes) return;
    int K = node_union(n, ptr, inc, col_conn, npe_col, ne, sbuf[w], suni[w], lane);
    if (K < 0 || K > kMaxAdjacency) return;
    int64_t a0 = adj_ptr[n];
    for (int i = lane; i < K; i += 32) adj[a0 + i] = suni[w][i];
    int64_t b = ptr[n];
    int m = (int)(ptr[n + 1] - b);
    for (int i = lane; i < m * npe_col; i += 32) {
        int k = i / npe_col, j = i - k * npe_col;
        uint32_t e = inc[b + k] >> 4;
        int32_t v = col_conn[(int64_t)j * ne + e];
        int lo = 0, hi = K - 1;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (suni[w][mid] < v) lo = mid + 1; else hi = mid;
        }
        slots[(b + k) * kSlotStride + slot_off + j] = (uint8_t)lo;
    }
    if (slot_off == 0)  // the row node's local index, for the row kernels' staged slot maps
        for (int k = lane; k < m; k += 32) slots[(b + k) * kSlotStride + kSlotLocal] = (uint8_t)(inc[b + k] & 15u);
}

__global__ void k_csr(const int64_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj, int64_t nnodes,
                      int dr_n, int dc_n, int64_t *rowptr, int32_t *colind, int64_t nnz) {
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t n = blockIdx.x * (int64_t)(blockDim.x >> 5) + w;
    if (n >= nnodes) return;
    int64_t a0 = adj_ptr[n];
    int K = (int)(adj_ptr[n + 1] - a0);
    int64_t base = (int64_t)dr_n * dc_n * a0;
    if (lane < dr_n) rowptr[n * dr_n + lane] = base + (int64_t)lane * dc_n * K;
    if (n == nnodes - 1 && lane == 0) rowptr[nnodes * dr_n] = nnz;
    for (int i = lane; i < K * dc_n; i += 32) {
        int s = i / dc_n, dc = i - s * dc_n;
        int32_t c = adj[a0 + s] * dc_n + dc;
        for (int dr = 0; dr < dr_n; dr++) colind[base + (int64_t)dr * dc_n * K + i] = c;
    }
}

// ---- scans ------------------------------------------------------------
template <class TIn>
__global__ void k_scan_block(const TIn *in, int64_t *out, int64_t *bsum, int64_t n) {
    __shared__ int64_t ws[32];
    int64_t i = blockIdx.x * 1024LL + threadIdx.x;
    int64_t v = i < n ? (int64_t)in[i] : 0;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    int64_t incl = x + (w > 0 ? ws[w - 1] : 0);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == 1023 && bsum) bsum[blockIdx.x] = incl;
}

__global__ void k_scan_add(int64_t *out, const int64_t *boff, int64_t n) {
    int64_t i = blockIdx.x * 1024LL + threadIdx.x;
    if (i < n) out[i] += boff[blockIdx.x];
}

template <class TIn>
void scan_impl(const TIn *in, int64_t *out, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    int64_t nb = (n + 1023) / 1024;
    if (nb == 1) {
        k_scan_block<TIn><<<1, 1024, 0, s>>>(in, out, nullptr, n);
        return;
    }
    DBuf<int64_t> bsum, boff;
    bsum.alloc(nb);
    boff.alloc(nb);
    k_scan_block<TIn><<<(unsigned)nb, 1024, 0, s>>>(in, out, bsum.p, n);
    scan_impl<int64_t>(bsum.p, boff.p, nb, s);
    k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(out, boff.p, n);
    FEDD_CUDA(cudaStreamSynchronize(s));  // temporaries die at scope exit
}

}  // namespace

void exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s) {
    scan_impl<int64_t>(in, out, n, s);
}
void exclusive_scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, cudaStream_t s) {
    scan_impl<int32_t>(in, out, n, s);
}

static int64_t read_i64(const int64_t *d, cudaStream_t s) {
    int64_t v = 0;
    FEDD_CUDA(cudaMemcpyAsync(&v, d, sizeof v, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    return v;
}

static void check_err(int *d_err, cudaStream_t s, const char *what) {
    int e = 0;
    FEDD_CUDA(cudaMemcpyAsync(&e, d_err, sizeof e, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    if (e == kDevMesh) FEDD_FAIL(FEDD_ERR_MESH, std::string(what) + ": element node index out of range");
    if (e == kDevCapacity)
        FEDD_FAIL(FEDD_ERR_CAPACITY, std::string(what) + ": a node exceeds " + std::to_string(kMaxIncidence) +
                                         " incident elements or " + std::to_string(kMaxAdjacency) + " neighbours");
    if (e) FEDD_FAIL(FEDD_ERR_CUDA, std::string(what) + ": device error " + std::to_string(e));
}

// node-level adjacency count + fill for a given incidence structure
static void adjacency(int64_t nnodes, const int64_t *ptr, const uint32_t *inc, int64_t ne, const int32_t *col_conn,
                      int npe_col, int slot_off, uint8_t *slots, DBuf<int64_t> &adj_ptr, DBuf<int32_t> &adj,
                      int &max_adj, int64_t &n_adj, int *d_err, cudaStream_t s) {
    DBuf<int64_t> cnt;
    DBuf<int> dmax;
    cnt.alloc(nnodes + 1);
    cnt.zero(s);
    dmax.alloc(1);
    dmax.zero(s);
    unsigned nb = ceil_div(nnodes, kGraphWarps);
    k_adj_count<<<nb, 32 * kGraphWarps, 0, s>>>(ptr, inc, col_conn, npe_col, ne, nnodes, cnt.p, d_err, dmax.p);
    FEDD_CUDA(cudaGetLastError());
    check_err(d_err, s, "adjacency");
    adj_ptr.alloc(nnodes + 1);
    exclusive_scan_i64(cnt.p, adj_ptr.p, nnodes + 1, s);
    n_adj = read_i64(adj_ptr.p + nnodes, s);
    int mx = 0;
    FEDD_CUDA(cudaMemcpyAsync(&mx, dmax.p, sizeof mx, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    max_adj = mx;
    adj.alloc(n_adj > 0 ? n_adj : 1);
    k_adj_fill<<<nb, 32 * kGraphWarps, 0, s>>>(ptr, inc, col_conn, npe_col, ne, nnodes, adj_ptr.p, adj.p, slots,
                                                slot_off);
    FEDD_CUDA(cudaGetLastError());
    FEDD_CUDA(cudaStreamSynchronize(s));
}

void build_graph(Graph &g, int64_t ne, const int32_t *row_conn, int npe_row, int64_t nrow_nodes,
                 const int32_t *col_conn, int npe_col, int64_t ncol_nodes, int slot_off, int *d_err,
                 cudaStream_t s) {
    g.nrow_nodes = nrow_nodes;
    g.ncol_nodes = ncol_nodes;
    DBuf<int32_t> cnt, cursor;
    DBuf<int> dmax;
    cnt.alloc(nrow_nodes + 1);
    cnt.zero(s);
    cursor.alloc(nrow_nodes);
    cursor.zero(s);
    dmax.alloc(1);
    dmax.zero(s);
    int64_t nt = ne * npe_row;
    k_count_inc<<<ceil_div(nt, 256), 256, 0, s>>>(row_conn, npe_row, ne, nrow_nodes, cnt.p, d_err);
    FEDD_CUDA(cudaGetLastError());
    check_err(d_err, s, "incidence count");
    g.inc_ptr.alloc(nrow_nodes + 1);
    exclusive_scan_i32_to_i64(cnt.p, g.inc_ptr.p, nrow_nodes + 1, s);
    g.n_inc = read_i64(g.inc_ptr.p + nrow_nodes, s);
    g.inc.alloc(g.n_inc);
    k_fill_inc<<<ceil_div(nt, 256), 256, 0, s>>>(row_conn, npe_row, ne, nrow_nodes, g.inc_ptr.p, cursor.p, g.inc.p);
    k_sort_inc<<<ceil_div(nrow_nodes, 128), 128, 0, s>>>(g.inc_ptr.p, g.inc.p, nrow_nodes, d_err, dmax.p);
    FEDD_CUDA(cudaGetLastError());
    check_err(d_err, s, "incidence sort");
    FEDD_CUDA(cudaMemcpyAsync(&g.max_inc, dmax.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    g.slots.alloc(g.n_inc * kSlotStride);
    g.slots.zero(s);
    adjacency(nrow_nodes, g.inc_ptr.p, g.inc.p, ne, col_conn, npe_col, slot_off, g.slots.p, g.adj_ptr, g.adj,
              g.max_adj, g.n_adj, d_err, s);
}

void build_graph_extra(const Graph &g, int64_t ne, const int32_t *col_conn, int npe_col, int64_t ncol_nodes,
                       int slot_off, DBuf<int64_t> &adj2_ptr, DBuf<int32_t> &adj2, int &max_adj2, int64_t &n_adj2,
                       int *d_err, cudaStream_t s) {
    (void)ncol_nodes;
    adjacency(g.nrow_nodes, g.inc_ptr.p, g.inc.p, ne, col_conn, npe_col, slot_off, g.slots.p, adj2_ptr, adj2,
              max_adj2, n_adj2, d_err, s);
}

// ---- Taylor-Hood vertex map ------------------------------------------------
__global__ void k_vmap_fill(const int32_t *__restrict__ conn2, const int32_t *__restrict__ conn1, int64_t ne,
                            int32_t *vmap) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    for (int k = 0; k < 4; k++) vmap[conn2[k * ne + e]] = conn1[k * ne + e];
}

__global__ void k_vmap_check_elems(const int32_t *__restrict__ conn2, const int32_t *__restrict__ conn1, int64_t ne,
                                   const int32_t *__restrict__ vmap, int *bad) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    for (int k = 0; k < 4; k++)
        if (vmap[conn2[k * ne + e]] != conn1[k * ne + e]) atomicOr(bad, 1);
    for (int k = 4; k < 10; k++)
        if (vmap[conn2[k * ne + e]] >= 0) atomicOr(bad, 2);
}

__global__ void k_vmap_count(const int32_t *__restrict__ vmap, int64_t nn2, int64_t nn1, int *cnt, int *bad) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nn2) return;
    const int32_t q = vmap[v];
    if (q >= nn1) atomicOr(bad, 4);
    else if (q >= 0) atomicAdd(cnt + q, 1);
}

// one warp per P2 node: a mapped vertex has exactly one preimage of its P1
// node and the same adjacency row in both graphs
__global__ void k_vmap_rows(const int32_t *__restrict__ vmap, int64_t nn2, const int *__restrict__ cnt,
                            const int64_t *__restrict__ ap2, const int32_t *__restrict__ adj2,
                            const int64_t *__restrict__ ap1, const int32_t *__restrict__ adj1, int *bad) {
    const int64_t v = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (v >= nn2) return;
    const int32_t q = vmap[v];
    if (q < 0) return;
    const int64_t a2 = ap2[v], k2 = ap2[v + 1] - a2, a1 = ap1[q], k1 = ap1[q + 1] - a1;
    if (lane == 0 && (cnt[q] != 1 || k1 != k2)) atomicOr(bad, 8);
    if (k1 != k2) return;
    for (int64_t i = lane; i < k2; i += 32)
        if (adj2[a2 + i] != adj1[a1 + i]) atomicOr(bad, 16);
}

__global__ void k_vmap_cover(const int *__restrict__ cnt, int64_t nn1, int *bad) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q < nn1 && cnt[q] != 1) atomicOr(bad, 32);
}

bool build_vertex_map(const int32_t *conn2, const int32_t *conn1, int64_t ne, int64_t nn2, int64_t nn1,
                      const Graph &g2, const Graph &g1, DBuf<int32_t> &vmap, cudaStream_t s) {
    if (ne == 0 || nn2 == 0 || nn1 == 0) return false;
    vmap.alloc(nn2);
    FEDD_CUDA(cudaMemsetAsync(vmap.p, 0xff, nn2 * sizeof(int32_t), s));  // -1
    DBuf<int> cnt, bad;
    cnt.alloc(nn1);
    cnt.zero(s);
    bad.alloc(1);
    bad.zero(s);
    k_vmap_fill<<<ceil_div(ne, 256), 256, 0, s>>>(conn2, conn1, ne, vmap.p);
    k_vmap_check_elems<<<ceil_div(ne, 256), 256, 0, s>>>(conn2, conn1, ne, vmap.p, bad.p);
    k_vmap_count<<<ceil_div(nn2, 256), 256, 0, s>>>(vmap.p, nn2, nn1, cnt.p, bad.p);
    k_vmap_rows<<<ceil_div(nn2, 8), 256, 0, s>>>(vmap.p, nn2, cnt.p, g2.adj_ptr.p, g2.adj.p, g1.adj_ptr.p, g1.adj.p,
                                                  bad.p);
    k_vmap_cover<<<ceil_div(nn1, 256), 256, 0, s>>>(cnt.p, nn1, bad.p);
    FEDD_CUDA(cudaGetLastError());
    int b = 0;
    FEDD_CUDA(cudaMemcpyAsync(&b, bad.p, sizeof b, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    return b == 0;
}

// largest element index among the incidences of each node range
// [bounds[k], bounds[k + 1]); one warp per node, its range found by a scan
// of the K + 1 bounds
__global__ void k_range_max_elem(const int64_t *__restrict__ inc_ptr, const uint32_t *__restrict__ inc,
                                 const int64_t *__restrict__ bounds, int K, int *out) {
    const int64_t n = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (n >= bounds[K]) return;  // uniform per warp
    int m = -1;
    for (int64_t i = inc_ptr[n] + lane; i < inc_ptr[n + 1]; i += 32) m = max(m, (int)(inc[i] >> 4));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
        int k = 0;
        while (k + 1 < K && n >= bounds[k + 1]) k++;
        atomicMax(out + k, m);
    }
}

void node_range_max_elem(const Graph &g, const int64_t *bounds, int K, int64_t *out, cudaStream_t s) {
    DBuf<int64_t> db;
    DBuf<int> dm;
    db.upload(bounds, (size_t)K + 1, s);
    dm.alloc((size_t)K);
    FEDD_CUDA(cudaMemsetAsync(dm.p, 0xff, (size_t)K * sizeof(int), s));  // -1
    if (bounds[K] > 0) {
        k_range_max_elem<<<(unsigned)ceil_div(bounds[K] * 32, 256), 256, 0, s>>>(g.inc_ptr.p, g.inc.p, db.p, K, dm.p);
        FEDD_CUDA(cudaGetLastError());
    }
    std::vector<int> m((size_t)K);
    FEDD_CUDA(cudaMemcpyAsync(m.data(), dm.p, (size_t)K * sizeof(int), cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < K; k++) out[k] = m[(size_t)k];
}

void build_csr(Csr &c, const DBuf<int64_t> &adj_ptr, const DBuf<int32_t> &adj, int64_t nrow_nodes,
               int64_t ncol_nodes, int dofs_r, int dofs_c, cudaStream_t s) {
    int64_t n_adj = read_i64(adj_ptr.p + nrow_nodes, s);
    c.nrows = nrow_nodes * dofs_r;
    c.ncols = ncol_nodes * dofs_c;
    c.nnz = n_adj * dofs_r * dofs_c;
    c.rowptr.alloc(c.nrows + 1);
    c.colind.alloc(c.nnz > 0 ? c.nnz : 1);
    if (nrow_nodes > 0) {
        k_csr<<<ceil_div(nrow_nodes, 8), 256, 0, s>>>(adj_ptr.p, adj.p, nrow_nodes, dofs_r, dofs_c, c.rowptr.p,
                                                       c.colind.p, c.nnz);
        FEDD_CUDA(cudaGetLastError());
    }
    FEDD_CUDA(cudaStreamSynchronize(s));
}

}  // namespace fedd
