// k_bc.cu -- Dirichlet rows and right-hand sides on the device.
//
// BCBuilder::setSystem (feddlib/core/General/BCBuilder_def.hpp:590-618) and
// setDirichletBC / setLocalRowOne / setLocalRowZero (:620-700): every row of
// a Dirichlet dof becomes, in the diagonal block of its block row, zero except
// a one at its diagonal entry (a row whose pattern has no diagonal entry stays
// all zero), and zero in the off-diagonal blocks.  BCBuilder::setRHS (:93-200)
// and setBCMinusVector (:232-350): the right-hand side at a Dirichlet dof is
// the boundary value g, or g minus a given vector.
#include "kernels.cuh"

namespace fedd {
namespace {

// one warp per Dirichlet row; the row's values are contiguous in CSR order
__global__ void k_dirichlet_rows(const int64_t *__restrict__ rows, int64_t nrows, const int64_t *__restrict__ rowptr,
                                 const int32_t *__restrict__ colind, double *vals, int diagonal_block) {
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= nrows) return;
    const int64_t r = rows[wid];
    for (int64_t e = rowptr[r] + lane; e < rowptr[r + 1]; e += 32)
        vals[e] = (diagonal_block && colind[e] == r) ? 1.0 : 0.0;
}

__global__ void k_dirichlet_rhs(const int64_t *__restrict__ rows, int64_t n, const double *__restrict__ g,
                                const double *__restrict__ sub, double *res) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int64_t k = rows[t];
    res[k] = (g ? g[k] : 0.0) - (sub ? sub[k] : 0.0);
}

}  // namespace

void launch_dirichlet_rows(const int64_t *rows, int64_t nrows, const int64_t *rowptr, const int32_t *colind,
                           double *vals, bool diagonal_block, cudaStream_t s, LaunchCounter &lc) {
    if (nrows == 0 || !vals) return;
    k_dirichlet_rows<<<(unsigned)ceil_div(nrows * 32, 256), 256, 0, s>>>(rows, nrows, rowptr, colind, vals,
                                                                       diagonal_block ? 1 : 0);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

void launch_dirichlet_rhs(const int64_t *rows, int64_t n, const double *g, const double *sub, double *res,
                          cudaStream_t s, LaunchCounter &lc) {
    if (n == 0 || !res) return;
    k_dirichlet_rhs<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(rows, n, g, sub, res);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

}  // namespace fedd
