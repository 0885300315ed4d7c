// engine.hpp -- host-side structures shared by the engine's translation units.
#pragma once
#include "common.cuh"

namespace fedd {

// ------------------------------------------------------------- tables ----
// Quadrature rules and basis tables (feddlib/core/FE/Helper.cpp) evaluated
// once on the host in FP64.  Rules: 1, 4 (AceGen code 18), 5, 15 points.
struct Rule {
    int n = 0;
    double pts[15][3];
    double w[15];
};
Rule make_rule(int npts);
void basis_phi(int order, const double *p, double *v);    // Helper::phi, 3D
void basis_dphi(int order, const double *p, double *g);   // Helper::gradPhi, 3D

// Navier-Stokes reference tensors for affine P2-P1 elements (exact integrals
// over the reference tetrahedron, evaluated with the reference's 15- and
// 5-point rules):
//   KS[a][b][s]    = sum_q w_q dc phi_a dd phi_b, s over (00,11,22,01+10,02+20,12+21)
//   T[c][a][b][k]  = sum_q w_q phi_a phi_k dc phi_b        (advection)
//   R[a][b][m]     = sum_q w_q lambda_m phi_a phi_b          (Newton term)
//   Y[c][p][b]     = sum_q5 w_q psi_p dc phi_b               (divergence)
//   DV[m][k][c]    = dc phi_k at vertex m                    (grad u at vertices)
//   WPHI, DQ, PHIQ = weights x basis, reference gradients and basis at the
//                    15 points (advection evaluated at the quadrature points)
struct NSTables {
    float KS[10][10][6];
    float T[3][10][10][10];
    float R[10][10][4];
    float Y[3][4][10];
    float DV[4][10][3];
    // quadrature-point form of the advection term (15-point rule):
    float WPHI[10][16];    // w_q phi_a(q)
    float DQ[10][3][16];   // d_c phi_b(q) (reference gradients)
    float PHIQ[15][10];    // phi_k(q)
};
void make_ns_tables(NSTables *t);

// Hyperelastic tables: reference P2 gradients and weights at the rule.
struct HyperTables {
    int nq;
    float w[5];
    float dphi[5][10][3];
};
void make_hyper_tables(int npts, HyperTables *t);

// ------------------------------------------------------------- graph -----
// Node -> element incidence plus the sorted node adjacency of one block.
// For a row node n: incidences inc[inc_ptr[n] .. inc_ptr[n+1]) packed as
// (element << 4) | local_row_index, ascending; per incidence kSlotStride
// bytes: slot (position in adj row of n) of each of the element's column
// nodes, at byte offset `slot_off`.
struct Graph {
    int64_t nrow_nodes = 0, ncol_nodes = 0;
    DBuf<int64_t> inc_ptr;   // nrow_nodes + 1
    DBuf<uint32_t> inc;      // incidences
    DBuf<uint8_t> slots;     // incidences * kSlotStride
    DBuf<int64_t> adj_ptr;   // nrow_nodes + 1
    DBuf<int32_t> adj;       // neighbour node ids, ascending per row node
    int max_inc = 0, max_adj = 0;
    int64_t n_inc = 0, n_adj = 0;
};

// Builds incidences of `row_conn` (SoA, npe_row x ne) and the adjacency
// towards `col_conn` (SoA, npe_col x ne).  Slots land at `slot_off`.
void build_graph(Graph &g, int64_t ne, const int32_t *row_conn, int npe_row, int64_t nrow_nodes,
                 const int32_t *col_conn, int npe_col, int64_t ncol_nodes, int slot_off,
                 int *d_err, cudaStream_t s);
// Adds a second adjacency (e.g. velocity rows -> pressure columns) that
// reuses g's incidences: fills adj2/adj2_ptr and slots at slot_off.
void build_graph_extra(const Graph &g, int64_t ne, const int32_t *col_conn, int npe_col,
                       int64_t ncol_nodes, int slot_off, DBuf<int64_t> &adj2_ptr,
                       DBuf<int32_t> &adj2, int &max_adj2, int64_t &n_adj2, int *d_err,
                       cudaStream_t s);

// CSR of a block whose rows are (row node, dr) for dr < dofs_r and whose
// columns are (adjacent node, dc) for dc < dofs_c, node-wise numbering.
struct Csr {
    int64_t nrows = 0, ncols = 0, nnz = 0;
    DBuf<int64_t> rowptr;
    DBuf<int32_t> colind;
};
void build_csr(Csr &c, const DBuf<int64_t> &adj_ptr, const DBuf<int32_t> &adj, int64_t nrow_nodes,
               int64_t ncol_nodes, int dofs_r, int dofs_c, cudaStream_t s);

// Taylor-Hood vertex map: vmap[v] = the P1 node at P2 vertex v (-1 for edge
// nodes), built from the elements' first four P2 nodes and the P1 element
// nodes at the same local positions.  Returns true when the map is
// consistent element by element, one-to-one onto the P1 nodes, no mapped
// node appears at an edge position, and each mapped vertex's adjacency row in
// g2 equals its P1 node's row in g1: the velocity-row kernel may then
// assemble the pressure rows of the vertices as well.
bool build_vertex_map(const int32_t *conn2, const int32_t *conn1, int64_t ne, int64_t nn2, int64_t nn1,
                      const Graph &g2, const Graph &g1, DBuf<int32_t> &vmap, cudaStream_t s);

// For K node ranges [bounds[k], bounds[k + 1]) of g's row nodes (bounds on
// the host): the largest element index among each range's incidences (-1 for
// none) into out[K] on the host.  Synchronises s.
void node_range_max_elem(const Graph &g, const int64_t *bounds, int K, int64_t *out, cudaStream_t s);

// element arrays: num_elements x npe (AoS, as the C ABI takes them) to the
// npe x num_elements layout the graph build reads, on the device
void device_aos_to_soa(const int32_t *aos, int64_t ne, int npe, int32_t *soa, cudaStream_t s);

// message slot of handle-less C-ABI calls (per host thread)
std::string &thread_error();

// exclusive scan helpers (device)
void exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s);
void exclusive_scan_i32_to_i64(const int32_t *in, int64_t *out, int64_t n, cudaStream_t s);

}  // namespace fedd
