// k_rhs.cu -- FE::assemblyRHS with a source function, FP64 throughout.
//
// FE::assemblyRHS (feddlib/core/FE/FE_def.hpp:7303-7400) evaluates the
// source at the physical quadrature points of each element,
//     x_q = B xhat_q + x_0,   B = [x_1 - x_0, x_2 - x_0, x_3 - x_0],
// on the rule Helper::determineDegree(dim, FEType, Std) selects (1 point for
// P1, 5 points for P2), and adds
//     b[(node of a) c] += |det B| sum_q w_q phi_a(q) f_c(x_q)
// for fieldType "Scalar" (c = 0) and "Vector" (node-wise dofs, c = 0..2).
// The caller evaluates its function at the points k_rhs_points hands out;
// k_rhs_elem forms the element contributions and k_rhs_rows sums them per
// node over the node's incidences in ascending element order.
#include "kernels.cuh"

namespace fedd {
namespace {

__device__ __forceinline__ void rhs_geometry(const double *__restrict__ xyz, const int32_t *__restrict__ conn,
                                             int64_t ne, int64_t e, double B[9], double x0[3]) {
    const int32_t n0 = conn[e], n1 = conn[ne + e], n2 = conn[2 * ne + e], n3 = conn[3 * ne + e];
    for (int j = 0; j < 3; j++) {
        x0[j] = xyz[3 * (int64_t)n0 + j];
        B[3 * j] = xyz[3 * (int64_t)n1 + j] - x0[j];
        B[3 * j + 1] = xyz[3 * (int64_t)n2 + j] - x0[j];
        B[3 * j + 2] = xyz[3 * (int64_t)n3 + j] - x0[j];
    }
}

__global__ void k_rhs_points(const double *__restrict__ xyz, const int32_t *__restrict__ conn, int64_t ne,
                             RhsRule R, double *xq) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double B[9], x0[3];
    rhs_geometry(xyz, conn, ne, e, B, x0);
    for (int q = 0; q < R.nq; q++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;  // in the reference's order: sum_k B[j][k] xhat[k], then x_0
            for (int k = 0; k < 3; k++) s = __dadd_rn(s, __dmul_rn(B[3 * j + k], R.xhat[q][k]));
            xq[(e * R.nq + q) * 3 + j] = __dadd_rn(s, x0[j]);
        }
}

// per element and local node a: |det B| sum_q w_q phi_a(q) f_c(x_q)
__global__ void k_rhs_elem(const double *__restrict__ xyz, const int32_t *__restrict__ conn, int64_t ne,
                           RhsRule R, const double *__restrict__ fq, int ncomp, double *stage, int *err) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double B[9], x0[3];
    rhs_geometry(xyz, conn, ne, e, B, x0);
    const double det = B[0] * (B[4] * B[8] - B[5] * B[7]) - B[1] * (B[3] * B[8] - B[5] * B[6]) +
                       B[2] * (B[3] * B[7] - B[4] * B[6]);
    if (!(det != 0.0) || !isfinite(det)) set_dev_error(err, kDevBadDet);
    const double ad = fabs(det);
    const double *f = fq + e * R.nq * ncomp;
    double *S = stage + e * R.npe * ncomp;
    for (int a = 0; a < R.npe; a++)
        for (int c = 0; c < ncomp; c++) {
            double v = 0.0;
            for (int q = 0; q < R.nq; q++)  // (w_q phi_a(q)) f, summed, then |det B|, rounded as written
                v = __dadd_rn(v, __dmul_rn(__dmul_rn(R.w[q], R.phi[q][a]), f[q * ncomp + c]));
            S[a * ncomp + c] = __dmul_rn(v, ad);
        }
}

// per node: the sum over its incidences, ascending element order
__global__ void k_rhs_rows(const int64_t *__restrict__ inc_ptr, const uint32_t *__restrict__ inc, int64_t nn,
                           const double *__restrict__ stage, int npe, int ncomp, double *rhs) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t t = inc_ptr[n]; t < inc_ptr[n + 1]; t++) {
        const uint32_t ea = inc[t];
        const double *S = stage + ((int64_t)(ea >> 4) * npe + (ea & 15u)) * ncomp;
        for (int c = 0; c < ncomp; c++) acc[c] += S[c];
    }
    for (int c = 0; c < ncomp; c++) rhs[n * ncomp + c] = acc[c];
}

}  // namespace

RhsRule make_rhs_rule(int order) {
    RhsRule R{};
    const Rule q = make_rule(order == 1 ? 1 : 5);
    R.nq = q.n;
    R.npe = order == 1 ? 4 : 10;
    for (int k = 0; k < q.n; k++) {
        for (int j = 0; j < 3; j++) R.xhat[k][j] = q.pts[k][j];
        R.w[k] = q.w[k];
        basis_phi(order, q.pts[k], R.phi[k]);
    }
    return R;
}

void launch_rhs_points(const double *xyz, const int32_t *conn, int64_t ne, const RhsRule &R, double *xq,
                       cudaStream_t s) {
    if (ne == 0) return;
    k_rhs_points<<<(unsigned)ceil_div(ne, 128), 128, 0, s>>>(xyz, conn, ne, R, xq);
    FEDD_CUDA(cudaGetLastError());
}

void launch_rhs_assemble(const Graph &g, const double *xyz, const int32_t *conn, int64_t ne, const RhsRule &R,
                         const double *fq, int ncomp, double *stage, double *rhs, int *d_err, cudaStream_t s) {
    if (ne > 0) {
        k_rhs_elem<<<(unsigned)ceil_div(ne, 128), 128, 0, s>>>(xyz, conn, ne, R, fq, ncomp, stage, d_err);
        FEDD_CUDA(cudaGetLastError());
    }
    if (g.nrow_nodes > 0) {
        k_rhs_rows<<<(unsigned)ceil_div(g.nrow_nodes, 128), 128, 0, s>>>(g.inc_ptr.p, g.inc.p, g.nrow_nodes, stage,
                                                                        R.npe, ncomp, rhs);
        FEDD_CUDA(cudaGetLastError());
    }
}

}  // namespace fedd
