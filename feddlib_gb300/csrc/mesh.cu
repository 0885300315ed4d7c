// mesh.cu -- the mesh front end on the device:
//   * FEDDLib's structured unit-cube tetrahedral mesh (MeshStructured::
//     buildMesh3D, feddlib/core/Mesh/MeshStructured_def.hpp:622-1010, with the
//     orientation fix of Mesh::correctElementOrientation / flipElement,
//     Mesh_def.hpp:543-577, 648-735), bit-identical to the host generator in
//     gen.cpp;
//   * the P2 mesh of a P1 tetrahedral mesh (MeshUnstructured::
//     buildP2ofP1MeshEdge, feddlib/core/Mesh/MeshUnstructured_def.hpp:122-233);
//   * the element-array transpose the assembler's graph build consumes,
// so a large mesh is made, refined and assembled without a host round trip.
#include <vector>

#include "../../include/feddgpu.h"
#include "engine.hpp"

namespace fedd {
namespace {

// ---- structured generator ---------------------------------------------------
// draw n (0-based) of the host generator's splitmix64 stream from `seed`
__device__ __forceinline__ double unit_at(uint64_t seed, uint64_t n) {
    uint64_t z = seed + (n + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// the reference's six tetrahedra per hex, as lattice offsets (in half steps
// of the P2 lattice) of their vertices, and the P2 local edge order
__constant__ int c_tet[6][4][3] = {
    {{2, 0, 0}, {0, 0, 0}, {2, 0, 2}, {2, 2, 2}}, {{0, 0, 2}, {0, 0, 0}, {2, 0, 2}, {2, 2, 2}},
    {{2, 0, 0}, {0, 0, 0}, {2, 2, 0}, {2, 2, 2}}, {{0, 0, 0}, {0, 2, 0}, {2, 2, 0}, {2, 2, 2}},
    {{0, 0, 0}, {0, 2, 0}, {0, 2, 2}, {2, 2, 2}}, {{0, 0, 0}, {0, 0, 2}, {0, 2, 2}, {2, 2, 2}}};
__constant__ int c_edge[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};

__global__ void k_lattice(int M, int order, double *xyz) {
    const int P = order == 1 ? M + 1 : 2 * M + 1;
    const int64_t n = (int64_t)P * P * P;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = (int)(i % P), s = (int)((i / P) % P), t = (int)(i / ((int64_t)P * P));
    const double h = 1.0 / M;
    if (order == 1) {
        xyz[3 * i] = __dmul_rn(r, h);
        xyz[3 * i + 1] = __dmul_rn(s, h);
        xyz[3 * i + 2] = __dmul_rn(t, h);
    } else {
        xyz[3 * i] = __ddiv_rn(__dmul_rn(r, h), 2.0);
        xyz[3 * i + 1] = __ddiv_rn(__dmul_rn(s, h), 2.0);
        xyz[3 * i + 2] = __ddiv_rn(__dmul_rn(t, h), 2.0);
    }
}

// one thread per hex: its six elements in the reference's order
__global__ void k_hex_elems(int M, int order, int32_t *conn) {
    const int64_t nh = (int64_t)M * M * M;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nh) return;
    const int r = (int)(c % M), s = (int)((c / M) % M), t = (int)(c / ((int64_t)M * M));
    if (order == 1) {
        const int64_t n1 = M + 1;
        for (int k = 0; k < 6; k++)
            for (int v = 0; v < 4; v++)
                conn[24 * c + 4 * k + v] = (int32_t)((r + c_tet[k][v][0] / 2) + n1 * (s + c_tet[k][v][1] / 2) +
                                                     n1 * n1 * (t + c_tet[k][v][2] / 2));
    } else {
        const int64_t P = 2 * M + 1, PP = P * P;
        const int64_t x0 = 2 * r, y0 = 2 * s, z0 = 2 * t;
        for (int k = 0; k < 6; k++) {
            int32_t *e = conn + 60 * c + 10 * k;
            for (int v = 0; v < 4; v++)
                e[v] = (int32_t)(x0 + c_tet[k][v][0] + P * (y0 + c_tet[k][v][1]) + PP * (z0 + c_tet[k][v][2]));
            for (int m = 0; m < 6; m++) {
                const int *A = c_tet[k][c_edge[m][0]], *B = c_tet[k][c_edge[m][1]];
                e[4 + m] = (int32_t)(x0 + (A[0] + B[0]) / 2 + P * (y0 + (A[1] + B[1]) / 2) + PP * (z0 + (A[2] + B[2]) / 2));
            }
        }
    }
}

// interior P1 vertices move by (2u - 1) amp h per coordinate, draws 3k..3k+2
// for the k-th interior vertex in lattice order (the host's stream order);
// rounded operations only, as the host computes them
__global__ void k_jitter(int M, int order, uint64_t seed, double amp, double *xyz) {
    const int64_t ni = (int64_t)(M - 1) * (M - 1) * (M - 1);
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ni) return;
    const int r = 1 + (int)(k % (M - 1)), s = 1 + (int)((k / (M - 1)) % (M - 1)),
              t = 1 + (int)(k / ((int64_t)(M - 1) * (M - 1)));
    const double h = 1.0 / M;
    const int64_t n1 = M + 1, P = 2 * M + 1;
    const int64_t idx = order == 1 ? r + n1 * s + n1 * n1 * t : 2 * r + P * 2 * s + P * P * 2 * t;
    for (int d = 0; d < 3; d++) {
        const double u = unit_at(seed, 3 * (uint64_t)k + d);
        const double dx = __dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(2.0, u), 1.0), amp), h);
        xyz[3 * idx + d] = __dadd_rn(xyz[3 * idx + d], dx);
    }
}

// P2 edge nodes at the midpoints of their (jittered) vertices
__global__ void k_midpoints(const int32_t *__restrict__ conn, int64_t ne, double *xyz) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int32_t *ce = conn + 10 * e;
    for (int k = 0; k < 6; k++)
        for (int d = 0; d < 3; d++)
            xyz[3 * (int64_t)ce[4 + k] + d] = __dmul_rn(
                0.5, __dadd_rn(xyz[3 * (int64_t)ce[c_edge[k][0]] + d], xyz[3 * (int64_t)ce[c_edge[k][1]] + d]));
}

// det B by the rule of Sarrus with the host's operation order; a negative
// determinant flips the element (1<->2, and 4<->6, 8<->9 for P2)
__global__ void k_orient(const double *__restrict__ xyz, int64_t ne, int npe, int32_t *conn) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int32_t *c = conn + npe * e;
    const double *x0 = xyz + 3 * (int64_t)c[0];
    double v[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) v[3 * i + j] = __dsub_rn(xyz[3 * (int64_t)c[j + 1] + i], x0[i]);
    double d = __dmul_rn(__dmul_rn(v[0], v[4]), v[8]);
    d = __dadd_rn(d, __dmul_rn(__dmul_rn(v[1], v[5]), v[6]));
    d = __dadd_rn(d, __dmul_rn(__dmul_rn(v[2], v[3]), v[7]));
    d = __dsub_rn(d, __dmul_rn(__dmul_rn(v[6], v[4]), v[2]));
    d = __dsub_rn(d, __dmul_rn(__dmul_rn(v[7], v[5]), v[0]));
    d = __dsub_rn(d, __dmul_rn(__dmul_rn(v[8], v[3]), v[1]));
    if (d < 0) {
        int32_t tmp = c[1]; c[1] = c[2]; c[2] = tmp;
        if (npe == 10) {
            tmp = c[4]; c[4] = c[6]; c[6] = tmp;
            tmp = c[8]; c[8] = c[9]; c[9] = tmp;
        }
    }
}

// ---- P2 of P1 -----------------------------------------------------------------
// The edges of vertex v are its adjacency entries w > v (adjacency rows are
// sorted, so (v, w) runs in the lexicographic order of the reference's
// sorted unique edge list).  first_above: index of the first entry > v.
__device__ __forceinline__ int64_t first_above(const int32_t *adj, int64_t lo, int64_t hi, int32_t v) {
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (adj[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void k_edge_count(const int64_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj, int64_t nn,
                             int64_t *cnt) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v > nn) return;
    if (v == nn) {
        cnt[v] = 0;
        return;
    }
    cnt[v] = adj_ptr[v + 1] - first_above(adj, adj_ptr[v], adj_ptr[v + 1], (int32_t)v);
}

__global__ void k_edge_nodes(const int64_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj,
                             const int64_t *__restrict__ eoff, const double *__restrict__ xyz1, int64_t nn1,
                             double *xyz2) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nn1) return;
    for (int d = 0; d < 3; d++) xyz2[3 * v + d] = xyz1[3 * v + d];
    const int64_t a1 = adj_ptr[v + 1], f = first_above(adj, adj_ptr[v], a1, (int32_t)v);
    for (int64_t i = f; i < a1; i++) {
        const int64_t w = adj[i], id = nn1 + eoff[v] + (i - f);
        for (int d = 0; d < 3; d++) xyz2[3 * id + d] = 0.5 * (xyz1[3 * v + d] + xyz1[3 * w + d]);
    }
}

// P2 element e: the P1 vertices, then the node of edge (la, lb) at position
// 4=e01 5=e12 6=e02 7=e03 8=e13 9=e23 (determinePositionInElementP2)
__global__ void k_p2_elems(const int32_t *__restrict__ conn1, int64_t ne, const int64_t *__restrict__ adj_ptr,
                           const int32_t *__restrict__ adj, const int64_t *__restrict__ eoff, int64_t nn1,
                           int32_t *conn2, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int32_t v[4];
    for (int k = 0; k < 4; k++) v[k] = conn1[4 * e + k];
    for (int k = 0; k < 4; k++) conn2[10 * e + k] = v[k];
    for (int m = 0; m < 6; m++) {
        const int32_t a = v[c_edge[m][0]], b = v[c_edge[m][1]];
        const int32_t lo = a < b ? a : b, hi = a < b ? b : a;
        const int64_t f = first_above(adj, adj_ptr[lo], adj_ptr[lo + 1], lo);
        const int64_t i = first_above(adj, f, adj_ptr[lo + 1], hi - 1);  // first entry >= hi
        if (lo == hi || i >= adj_ptr[lo + 1] || adj[i] != hi) {
            set_dev_error(err, kDevMesh);
            conn2[10 * e + 4 + m] = 0;
            continue;
        }
        conn2[10 * e + 4 + m] = (int32_t)(nn1 + eoff[lo] + (i - f));
    }
}

__global__ void k_aos_to_soa(const int32_t *__restrict__ aos, int64_t ne, int npe, int32_t *soa) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ne * npe) return;
    const int64_t e = i / npe;
    const int a = (int)(i - e * npe);
    soa[(int64_t)a * ne + e] = aos[i];
}

}  // namespace

void device_aos_to_soa(const int32_t *aos, int64_t ne, int npe, int32_t *soa, cudaStream_t s) {
    if (ne == 0) return;
    k_aos_to_soa<<<(unsigned)ceil_div(ne * npe, 256), 256, 0, s>>>(aos, ne, npe, soa);
    FEDD_CUDA(cudaGetLastError());
}

}  // namespace fedd

// ---------------------------------------------------------------- C ABI ----
using namespace fedd;

struct fedd_p2mesh {
    int device = 0;
    int64_t nn1 = 0, nn2 = 0, ne = 0;
    DBuf<double> xyz2;
    DBuf<int32_t> conn2;
};

namespace {
// handle-less calls keep their message in the calling thread's slot, which
// fedd_last_error(NULL, ...) returns
template <class F> fedd_status run_guarded(F &&fn) {
    std::string &msg = thread_error();
    try {
        fn();
        msg.clear();
        return FEDD_OK;
    } catch (const Status &st) {
        msg = st.msg;
        return st.code;
    } catch (const CudaError &e) {
        msg = std::string(e.what) + ": " + cudaGetErrorString(e.code);
        return FEDD_ERR_CUDA;
    } catch (const std::bad_alloc &) {
        msg = "host allocation failed";
        return FEDD_ERR_NOMEM;
    } catch (...) {
        msg = "unexpected exception";
        return FEDD_ERR_CUDA;
    }
}
}  // namespace

extern "C" {

fedd_status fedd_mesh_structured_device(int32_t M, int32_t fe_order, uint64_t seed, double amp, double *coords,
                                        int32_t *elements, void *stream) {
    if (M < 1 || (fe_order != 1 && fe_order != 2) || !coords || !elements) return FEDD_ERR_ARG;
    if (6LL * M * M * M >= (1LL << 28)) return FEDD_ERR_ARG;
    return run_guarded([&] {
        cudaStream_t s = (cudaStream_t)stream;
        const int64_t P = fe_order == 1 ? M + 1 : 2 * M + 1, nn = P * P * P, ne = 6LL * M * M * M;
        const int npe = fe_order == 1 ? 4 : 10;
        k_lattice<<<(unsigned)ceil_div(nn, 256), 256, 0, s>>>(M, fe_order, coords);
        k_hex_elems<<<(unsigned)ceil_div((int64_t)M * M * M, 128), 128, 0, s>>>(M, fe_order, elements);
        if (amp != 0.0) {  // as the host generator: jitter, then midpoints recomputed from the vertices
            if (M > 1)
                k_jitter<<<(unsigned)ceil_div((int64_t)(M - 1) * (M - 1) * (M - 1), 256), 256, 0, s>>>(
                    M, fe_order, seed, amp, coords);
            if (fe_order == 2) k_midpoints<<<(unsigned)ceil_div(ne, 256), 256, 0, s>>>(elements, ne, coords);
        }
        k_orient<<<(unsigned)ceil_div(ne, 256), 256, 0, s>>>(coords, ne, npe, elements);
        FEDD_CUDA(cudaGetLastError());
        FEDD_CUDA(cudaStreamSynchronize(s));
    });
}

fedd_status fedd_p2_of_p1(int64_t num_nodes, int64_t num_elements, const double *coords, const int32_t *elements,
                          uint32_t flags, int device, fedd_p2mesh **out, int64_t *num_nodes_p2) {
    if (!out || !num_nodes_p2 || !coords || !elements || num_nodes <= 0 || num_elements <= 0) return FEDD_ERR_ARG;
    if (num_elements >= (1LL << 28) || num_nodes >= (1LL << 31)) return FEDD_ERR_ARG;
    *out = nullptr;
    fedd_p2mesh *m = new (std::nothrow) fedd_p2mesh;
    if (!m) return FEDD_ERR_NOMEM;
    fedd_status st = run_guarded([&] {
        FEDD_CUDA(cudaSetDevice(device));
        m->device = device;
        m->nn1 = num_nodes;
        m->ne = num_elements;
        cudaStream_t s = 0;
        const bool dev = flags & FEDD_MESH_DEVICE;
        DBuf<double> xyz1;
        DBuf<int32_t> aos, soa;
        const double *x1 = coords;
        const int32_t *c1 = elements;
        if (!dev) {
            xyz1.upload(coords, (size_t)num_nodes * 3, s);
            aos.upload(elements, (size_t)num_elements * 4, s);
            x1 = xyz1.p;
            c1 = aos.p;
        }
        soa.alloc((size_t)num_elements * 4);
        device_aos_to_soa(c1, num_elements, 4, soa.p, s);
        DBuf<int> err;
        err.alloc(1);
        err.zero(s);
        Graph g;
        build_graph(g, num_elements, soa.p, 4, num_nodes, soa.p, 4, num_nodes, 0, err.p, s);
        DBuf<int64_t> cnt, eoff;
        cnt.alloc(num_nodes + 1);
        eoff.alloc(num_nodes + 1);
        k_edge_count<<<(unsigned)ceil_div(num_nodes + 1, 256), 256, 0, s>>>(g.adj_ptr.p, g.adj.p, num_nodes, cnt.p);
        FEDD_CUDA(cudaGetLastError());
        exclusive_scan_i64(cnt.p, eoff.p, num_nodes + 1, s);
        int64_t nedges = 0;
        FEDD_CUDA(cudaMemcpyAsync(&nedges, eoff.p + num_nodes, sizeof nedges, cudaMemcpyDeviceToHost, s));
        FEDD_CUDA(cudaStreamSynchronize(s));
        m->nn2 = num_nodes + nedges;
        if (m->nn2 >= (1LL << 31)) FEDD_FAIL(FEDD_ERR_ARG, "P2 mesh exceeds 2^31 nodes");
        m->xyz2.alloc((size_t)m->nn2 * 3);
        m->conn2.alloc((size_t)num_elements * 10);
        k_edge_nodes<<<(unsigned)ceil_div(num_nodes, 256), 256, 0, s>>>(g.adj_ptr.p, g.adj.p, eoff.p, x1, num_nodes,
                                                                        m->xyz2.p);
        k_p2_elems<<<(unsigned)ceil_div(num_elements, 256), 256, 0, s>>>(c1, num_elements, g.adj_ptr.p, g.adj.p,
                                                                         eoff.p, num_nodes, m->conn2.p, err.p);
        FEDD_CUDA(cudaGetLastError());
        int e = 0;
        FEDD_CUDA(cudaMemcpyAsync(&e, err.p, sizeof e, cudaMemcpyDeviceToHost, s));
        FEDD_CUDA(cudaStreamSynchronize(s));
        if (e) FEDD_FAIL(FEDD_ERR_MESH, "P2 of P1: an element edge is missing from the node graph");
        *num_nodes_p2 = m->nn2;
    });
    if (st != FEDD_OK) {
        delete m;
        return st;
    }
    *out = m;
    return FEDD_OK;
}

fedd_status fedd_p2_copy(const fedd_p2mesh *m, double *coords, int32_t *elements, uint32_t flags) {
    if (!m) return FEDD_ERR_ARG;
    return run_guarded([&] {
        FEDD_CUDA(cudaSetDevice(m->device));
        const cudaMemcpyKind k = (flags & FEDD_MESH_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (coords) FEDD_CUDA(cudaMemcpy(coords, m->xyz2.p, (size_t)m->nn2 * 3 * sizeof(double), k));
        if (elements) FEDD_CUDA(cudaMemcpy(elements, m->conn2.p, (size_t)m->ne * 10 * sizeof(int32_t), k));
    });
}

fedd_status fedd_p2_destroy(fedd_p2mesh *m) {
    if (!m) return FEDD_ERR_ARG;
    cudaSetDevice(m->device);
    delete m;
    return FEDD_OK;
}

}  // extern "C"
