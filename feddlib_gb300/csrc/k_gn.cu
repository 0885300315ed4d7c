// k_gn.cu -- viscous part of the generalized-Newtonian Navier-Stokes element.
//
// AssembleFEGeneralizedNewtonian (feddlib/core/AceFemAssembly/specific/
// AssembleFEGeneralizedNewtonian_def.hpp) replaces the Newtonian Laplacian by
// the stress-divergence term with a shear-rate dependent viscosity:
//   S_(ak)(bl) = |det B| sum_q w_q eta(gamma_q) (d_kl g_a.g_b + g_a,l g_b,k)
//                (assemblyStress :225-416, degree 3 -> 5-point rule)
// and, with Newton, its derivative
//   D_(ak)(bl) = |det B| sum_q w_q (-2 c_q) G_b^l F_a^k
//                (assemblyStressDev :418-695, degree 4 -> 15-point rule)
// with c_q = -(2/gamma) d eta/d gamma, F_a^k = g_a . (row k of the symmetric
// velocity gradient) and G_b^l the same except for l = 3, where the
// reference's factor reads g_b,3 * (du_13 + du_31)/2 for the first term; it
// is restated as the reference computes it.  The residual's viscous part is
// S u = |det B| sum_q w_q eta sum_c g_a,c (du_kc + du_ck).  The rest of the
// element (advection, its Newton term, B and B^T) is the Navier-Stokes
// element, assembled by k_ns.cu with the Newtonian viscosity set to zero.
//
// One warp per element, elements taken in batches of 32 per warp; lane
// 3 b + l owns column (b, l) of the dense 30 x 30 matrix and row (b, l) of
// the residual.  Geometry is FP64, one element of the batch per lane; the
// rest is FP32.
#include <cmath>

#include "engine.hpp"
#include "kernels.cuh"

namespace fedd {
namespace {

struct GNTab {
    float w5[5];
    float d5[5][10][3];
    float w15[15];
    float d15[15][10][3];
};
__constant__ GNTab c_gn;

constexpr int kGNWarps = 4;

// FEDDLib's viscosity-model sources test abs(x) against small thresholds;
// with the headers they include that abs is the integer function, so the
// tests read |trunc(x)| (the Carreau-Yasuda a = 2 branch for every a in
// (1, 3), the shear-rate floor for every rate below 1).  Kept as the
// reference computes.
__device__ __forceinline__ float abs_int(float x) { return fabsf(truncf(x)); }

// CarreauYasuda_def.hpp:25-31, PowerLaw_def.hpp:27-44, Dimless_Carreau_def.hpp:26-31
__device__ float gn_eta(const ViscLaw &L, float g) {
    const float *c = L.prm;
    if (L.model == 0) return c[3] + (c[2] - c[3]) * powf(1.0f + powf(c[0] * g, c[4]), (c[1] - 1.0f) / c[4]);
    if (L.model == 1) {
        float eta = c[0] * powf(g, c[1] - 1.0f);
        if (eta < c[3])
            eta = c[3];
        else if (fabsf(eta) > c[2])
            eta = c[2];
        return eta;
    }
    return c[4] * (c[3] + (c[2] - c[3]) * powf(1.0f + (c[0] * g) * (c[0] * g), (c[1] - 1.0f) * 0.5f));
}

// -(2/gamma) d eta/d gamma: CarreauYasuda_def.hpp:39-57, PowerLaw_def.hpp:48-63,
// Dimless_Carreau_def.hpp:36-43
__device__ float gn_dterm(const ViscLaw &L, float g) {
    const float *c = L.prm;
    if (L.model == 0) {
        const float a = c[4];
        if (abs_int(a - 2.0f) < 2.220446049250313e-16f)
            return -2.0f * (c[2] - c[3]) * (c[1] - 1.0f) * powf(c[0], a) *
                   powf(1.0f + powf(c[0] * g, a), (c[1] - 1.0f - a) / a);
        if (abs_int(g) <= L.gamma_min) g = L.gamma_min;
        return -2.0f * (c[2] - c[3]) * (c[1] - 1.0f) * powf(c[0], a) * powf(g, a - 2.0f) *
               powf(1.0f + powf(c[0] * g, a), (c[1] - 1.0f - a) / a);
    }
    if (L.model == 1) {
        if (abs_int(g) <= L.gamma_min) g = L.gamma_min;
        return -2.0f * c[0] * (c[1] - 1.0f) * powf(g, c[1] - 3.0f);
    }
    return c[4] * (-2.0f * (c[2] - c[3]) * (c[1] - 1.0f) * c[0] * c[0] *
                   powf(1.0f + (c[0] * g) * (c[0] * g), (c[1] - 3.0f) * 0.5f));
}

// per-warp scratch: the element's velocities, and per quadrature point (5
// stress points, then 15 Newton points) the physical basis gradients, the
// stress points' gradients scaled by w eta and their w eta (du + du^T), and
// the Newton points' derivative weight, symmetric velocity gradient and row
// factors
constexpr int kGNRow = 44;  // 11 chunks of 16 B: the 16-byte stores of lanes q fall in different bank groups
struct __align__(16) GNWarpSmem {
    float su[32];
    float sg[20][kGNRow];   // sg[q][4 b + c] = d phi_b / d x_c at point q
    float sgw[5][kGNRow];   // stress points: w eta d phi_b / d x_c at 4 b + c
    float sT[5][6];         // stress points: w eta (du + du^T), entries 00 11 22 01 02 12
    float sw[20];           // Newton points (index 5 + q): -2 w c
    float sm[15][6];        // Newton points: du11, du22, du33, xy, xz, yz
    float sgeo[32][10];     // the batch's B^-1 (row-major) and |det B|, one row per element
    float sF[15][36];       // Newton points: F_a^k at index 3 a + k (rows 16-byte aligned)
};

__global__ void __launch_bounds__(32 * kGNWarps, 6) k_gn_elem(const double *__restrict__ xyz,
                                                          const int32_t *__restrict__ conn, int64_t ne,
                                                          const double *__restrict__ u, ViscLaw L, int newton,
                                                          float *stage, int *err, int64_t e_begin, int64_t e_end) {
    __shared__ GNWarpSmem smem[kGNWarps];
    // the rule tables in shared memory: phase 1 reads a different point per
    // lane, which constant memory would serialise
    __shared__ GNTab tab;
    for (int t = threadIdx.x; t < (int)(sizeof(GNTab) / sizeof(float)); t += blockDim.x)
        reinterpret_cast<float *>(&tab)[t] = reinterpret_cast<const float *>(&c_gn)[t];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    GNWarpSmem &S = smem[w];
    // Carreau-Yasuda takes its a = 2 formulas for every a in (1, 3) (see
    // abs_int): eta and the derivative term then share one power chain
    const bool cy2 = L.model == 0 && abs_int(L.prm[4] - 2.0f) < 2.220446049250313e-16f;
    const float e_eta = (L.prm[1] - 1.0f) / L.prm[4], e_dterm = (L.prm[1] - 1.0f - L.prm[4]) / L.prm[4];
    const float c0a = cy2 ? powf(L.prm[0], L.prm[4]) : 0.0f;
    for (int64_t e0 = e_begin + ((int64_t)blockIdx.x * kGNWarps + w) * 32; e0 < e_end;
         e0 += (int64_t)gridDim.x * kGNWarps * 32) {
        // FP64 geometry of a batch of 32 elements, one element per lane (the
        // FP64 pipe is narrow: one lane per element per warp would occupy it
        // 32 times as long)
        if (e0 + lane < e_end) {
            int32_t v[4];
            for (int k = 0; k < 4; k++) v[k] = conn[(int64_t)k * ne + e0 + lane];
            float gB[9];
            const float gdet = fabsf(d2f_rn(geometry_fp64(xyz, v[0], v[1], v[2], v[3], gB)));
            if (!(gdet > 0.0f) || !isfinite(gdet)) set_dev_error(err, kDevBadDet);
#pragma unroll
            for (int k = 0; k < 9; k++) S.sgeo[lane][k] = gB[k];
            S.sgeo[lane][9] = gdet;
        }
        __syncwarp();
        const int nb = (int)min((int64_t)32, e_end - e0);
#pragma unroll 1
        for (int t = 0; t < nb; t++) {
            const int64_t e = e0 + t;
            float Bi[9];
#pragma unroll
            for (int k = 0; k < 9; k++) Bi[k] = S.sgeo[t][k];
            const float adet = S.sgeo[t][9];
            const int b = lane < 30 ? lane / 3 : 0, l = lane < 30 ? lane - 3 * (lane / 3) : 0;
            if (lane < 30) S.su[lane] = d2f_rn(u[3 * (int64_t)conn[(int64_t)b * ne + e] + l]);
            __syncwarp();
            // phase 1: one lane per quadrature point (AssembleFEGeneralizedNewtonian_def.hpp:998-1083)
            const int nq = newton ? 20 : 5;
            if (lane < nq) {
                const int q = lane < 5 ? lane : lane - 5;
                const float(*d)[3] = lane < 5 ? tab.d5[q] : tab.d15[q];
                float g[30], du[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
                for (int k = 0; k < 10; k++) {
#pragma unroll
                    for (int c = 0; c < 3; c++) g[3 * k + c] = d[k][0] * Bi[c] + d[k][1] * Bi[3 + c] + d[k][2] * Bi[6 + c];
                    *reinterpret_cast<float4 *>(&S.sg[lane][4 * k]) = make_float4(g[3 * k], g[3 * k + 1], g[3 * k + 2], 0.0f);
#pragma unroll
                    for (int a1 = 0; a1 < 3; a1++)
#pragma unroll
                        for (int c = 0; c < 3; c++) du[3 * a1 + c] = fmaf(S.su[3 * k + a1], g[3 * k + c], du[3 * a1 + c]);
                }
                const float s01 = du[1] + du[3], s02 = du[2] + du[6], s12 = du[5] + du[7];
                const float gamma = sqrtf(2.0f * du[0] * du[0] + 2.0f * du[4] * du[4] + 2.0f * du[8] * du[8] + s01 * s01 +
                                          s02 * s02 + s12 * s12);
                // stress points: eta; Newton points: -(2/gamma) d eta/d gamma
                float lawv;
                if (cy2) {
                    // Carreau-Yasuda on the reference's a = 2 branch: both are
                    // (1 + (c0 gamma)^a)^e with e per lane, one power chain
                    // for all lanes instead of one per branch
                    const float *c = L.prm;
                    const float y = powf(1.0f + powf(c[0] * gamma, c[4]), lane < 5 ? e_eta : e_dterm);
                    lawv = lane < 5 ? c[3] + (c[2] - c[3]) * y : -2.0f * (c[2] - c[3]) * (c[1] - 1.0f) * c0a * y;
                } else {
                    lawv = lane < 5 ? gn_eta(L, gamma) : gn_dterm(L, gamma);
                }
                if (lane < 5) {
                    const float ew = lawv * tab.w5[q];
#pragma unroll
                    for (int k = 0; k < 10; k++)
                        *reinterpret_cast<float4 *>(&S.sgw[q][4 * k]) =
                            make_float4(ew * g[3 * k], ew * g[3 * k + 1], ew * g[3 * k + 2], 0.0f);
                    float *T = S.sT[q];
                    T[0] = ew * (2.0f * du[0]);
                    T[1] = ew * (2.0f * du[4]);
                    T[2] = ew * (2.0f * du[8]);
                    T[3] = ew * s01;
                    T[4] = ew * s02;
                    T[5] = ew * s12;
                } else {
                    S.sw[lane] = -2.0f * lawv * tab.w15[q];
                    const float xy = 0.5f * (du[1] + du[3]), xz = 0.5f * (du[6] + du[2]), yz = 0.5f * (du[7] + du[5]);
                    float *m = S.sm[q];
                    m[0] = du[0];
                    m[1] = du[4];
                    m[2] = du[8];
                    m[3] = xy;
                    m[4] = xz;
                    m[5] = yz;
#pragma unroll
                    for (int k = 0; k < 10; k++) {
                        const float g0 = g[3 * k], g1 = g[3 * k + 1], g2 = g[3 * k + 2];
                        S.sF[q][3 * k] = g0 * du[0] + g1 * xy + g2 * xz;
                        S.sF[q][3 * k + 1] = g0 * xy + g1 * du[4] + g2 * yz;
                        S.sF[q][3 * k + 2] = g0 * xz + g1 * yz + g2 * du[8];
                    }
                }
            }
            __syncwarp();
            // phase 2: lane 3 b + l accumulates column (b, l) and residual row (b, l);
            // lanes 30 and 31 keep zeros for the rows' two padding columns
            float acc[30];
#pragma unroll
            for (int p = 0; p < 30; p++) acc[p] = 0.0f;
            float r = 0.0f;
            if (lane < 30) {
                // stress: acc[(a, k)] += (w eta g_a).g_b d_kl + (w eta g_a,l) g_b,k
                const float e0 = l == 0 ? 1.0f : 0.0f, e1 = l == 1 ? 1.0f : 0.0f, e2 = l == 2 ? 1.0f : 0.0f;
                for (int q = 0; q < 5; q++) {
                    const float4 gb = *reinterpret_cast<const float4 *>(&S.sg[q][4 * b]);
                    const float4 *sw4 = reinterpret_cast<const float4 *>(S.sgw[q]);
#pragma unroll
                    for (int a = 0; a < 10; a++) {
                        const float4 s = sw4[a];
                        const float dot = s.x * gb.x + s.y * gb.y + s.z * gb.z;
                        const float sal = l == 0 ? s.x : (l == 1 ? s.y : s.z);
                        acc[3 * a] = fmaf(e0, dot, fmaf(sal, gb.x, acc[3 * a]));
                        acc[3 * a + 1] = fmaf(e1, dot, fmaf(sal, gb.y, acc[3 * a + 1]));
                        acc[3 * a + 2] = fmaf(e2, dot, fmaf(sal, gb.z, acc[3 * a + 2]));
                    }
                    // residual row (b, l): g_b . w eta (du + du^T)[l][:]
                    const float *T = S.sT[q];
                    const float t0 = l == 0 ? T[0] : (l == 1 ? T[3] : T[4]);
                    const float t1 = l == 0 ? T[3] : (l == 1 ? T[1] : T[5]);
                    const float t2 = l == 0 ? T[4] : (l == 1 ? T[5] : T[2]);
                    r = fmaf(gb.x, t0, fmaf(gb.y, t1, fmaf(gb.z, t2, r)));
                }
                if (newton) {
                    // G_b^l = g_b . (column l of the symmetric gradient: entries
                    // (0 3 4), (3 1 5), (4 5 2) of sm), except that for l = 2 the
                    // reference's factor takes g_b,3 in place of g_b,1 in the
                    // first term; per-lane indices instead of a branch on l
                    const int ip = l == 0 ? 0x430 : (l == 1 ? 0x513 : 0x254);  // i0 | i1 << 4 | i2 << 8
                    for (int q = 0; q < 15; q++) {
                        const float *m = S.sm[q];
                        const float4 gbn = *reinterpret_cast<const float4 *>(&S.sg[5 + q][4 * b]);
                        const float g0 = l == 2 ? gbn.z : gbn.x, g1 = gbn.y, g2 = gbn.z;
                        const float G = g0 * m[ip & 15] + g1 * m[(ip >> 4) & 15] + g2 * m[ip >> 8];
                        const float cg = S.sw[5 + q] * G;
                        const float4 *F4 = reinterpret_cast<const float4 *>(S.sF[q]);
#pragma unroll
                        for (int p4 = 0; p4 < 7; p4++) {
                            const float4 f = F4[p4];
                            acc[4 * p4] = fmaf(cg, f.x, acc[4 * p4]);
                            acc[4 * p4 + 1] = fmaf(cg, f.y, acc[4 * p4 + 1]);
                            acc[4 * p4 + 2] = fmaf(cg, f.z, acc[4 * p4 + 2]);
                            acc[4 * p4 + 3] = fmaf(cg, f.w, acc[4 * p4 + 3]);
                        }
                        const float2 f2 = reinterpret_cast<const float2 *>(S.sF[q])[14];
                        acc[28] = fmaf(cg, f2.x, acc[28]);
                        acc[29] = fmaf(cg, f2.y, acc[29]);
                    }
                }
            }
            // every lane stores, so each row goes out as a full 128 bytes (a
            // row with its padding unwritten leaves a partial 32-byte sector
            // that L2 would read back from DRAM to merge)
            float *Se = stage + e * kGNStride;
#pragma unroll
            for (int p = 0; p < 30; p++) Se[32 * p + lane] = acc[p] * adet;
            Se[kGNRes + lane] = r * adet;
            __syncwarp();  // the next element overwrites the scratch
        }
    }
}

// dense element matrices: adds the viscous part to the Navier-Stokes element
// matrices (34 x 34, velocity rows/columns first) of elements [first, first+count)
__global__ void k_gn_dense_add(const float *__restrict__ stage, int64_t first, int64_t count, double *Ke, double *re,
                               double cuu) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count * 930) return;
    const int64_t e = t / 930;
    const int k = (int)(t - e * 930);
    const float *S = stage + (first + e) * kGNStride;
    if (k < 900)
        Ke[e * 34 * 34 + (k / 30) * 34 + (k % 30)] += (double)S[32 * (k / 30) + k % 30];
    else
        re[e * 34 + (k - 900)] += cuu * (double)S[kGNRes + (k - 900)];  // the viscous residual is part of ANB_uu u
}

void upload_gn_tables(cudaStream_t s) {
    GNTab t{};
    Rule r5 = make_rule(5), r15 = make_rule(15);
    for (int q = 0; q < 5; q++) {
        double d[30];
        basis_dphi(2, r5.pts[q], d);
        t.w5[q] = (float)r5.w[q];
        for (int a = 0; a < 10; a++)
            for (int c = 0; c < 3; c++) t.d5[q][a][c] = (float)d[3 * a + c];
    }
    for (int q = 0; q < 15; q++) {
        double d[30];
        basis_dphi(2, r15.pts[q], d);
        t.w15[q] = (float)r15.w[q];
        for (int a = 0; a < 10; a++)
            for (int c = 0; c < 3; c++) t.d15[q][a][c] = (float)d[3 * a + c];
    }
    FEDD_CUDA(cudaMemcpyToSymbolAsync(c_gn, &t, sizeof t, 0, cudaMemcpyHostToDevice, s));
}

// ---- outflow Neumann boundary term ----------------------------------------
// AssembleFEGeneralizedNewtonian::assemblyOutflowNeumannBoundaryTerm
// (AssembleFEGeneralizedNewtonian_def.hpp:697-920) for an element flagged on
// face f, with the surface data FEDDLib's Domain attaches to a P2 face
// (setSurfaceNormalsForFE, setSurfaceQuadraturePointsWeights(flag, 8):
// Domain_def.hpp:1148-1255): n = unit((f0 - f1) x (f0 - f2)),
// s = |(f1 - f0) x (f2 - f0)|, the 7-point triangle rule x_q in barycentric
// form (Helper::getQuadraturePointsOnSurfaceInGlobalSpace, Helper.cpp:
// 1762-1893), mapped into the element's reference coordinates
// xi_q = B^-1 (x_q - x_0):
//   K[(i,d)][(j,e)] = -s sum_q eta(gamma_q) w_q (d phi_j / d x_d)(xi_q) n_e phi_i(xi_q).
// The reference adds K to the element's fixed-point matrix after its
// Jacobian has been formed from that matrix, so K reaches the residual,
//   r_(i,d) += -s sum_q eta_q w_q phi_i(xi_q) d/dx_d (u . n)(xi_q),
// and the matrix only as FE::assemblyNavierStokes' "FixedPoint" mode takes
// it (assembleFixedPoint's matrix, GNOutflow::matrix).  One warp per flagged
// element: every lane evaluates the point data, lane r < 30 owns residual
// row r and, for the matrix, column r = (j, e) summed over the points in
// registers; FP64 geometry, the rest FP32, added to the element's rows and
// residual row in the viscous stage, which the velocity rows fold in.
__device__ __forceinline__ void p2_basis_at(float x, float y, float z, float *phi, float *g) {
    // Helper::phi / Helper::gradPhi for P2 in 3D (Helper.cpp:503-590, 703-745);
    // local order 0-3 vertices, 4=e01, 5=e12, 6=e02, 7=e03, 8=e13, 9=e23
    const float l = 1.0f - x - y - z, t = -3.0f + 4.0f * x + 4.0f * y + 4.0f * z;
    phi[0] = l * (1.0f - 2.0f * x - 2.0f * y - 2.0f * z);
    phi[1] = x * (2.0f * x - 1.0f);
    phi[2] = y * (2.0f * y - 1.0f);
    phi[3] = z * (2.0f * z - 1.0f);
    phi[4] = 4.0f * x * l;
    phi[5] = 4.0f * x * y;
    phi[6] = 4.0f * y * l;
    phi[7] = 4.0f * z * l;
    phi[8] = 4.0f * x * z;
    phi[9] = 4.0f * y * z;
    const float G[30] = {t, t, t,
                         4.0f * x - 1.0f, 0.0f, 0.0f,
                         0.0f, 4.0f * y - 1.0f, 0.0f,
                         0.0f, 0.0f, 4.0f * z - 1.0f,
                         4.0f - 8.0f * x - 4.0f * y - 4.0f * z, -4.0f * x, -4.0f * x,
                         4.0f * y, 4.0f * x, 0.0f,
                         -4.0f * y, 4.0f - 4.0f * x - 8.0f * y - 4.0f * z, -4.0f * y,
                         -4.0f * z, -4.0f * z, 4.0f - 4.0f * x - 4.0f * y - 8.0f * z,
                         4.0f * z, 0.0f, 4.0f * x,
                         0.0f, 4.0f * z, 4.0f * y};
#pragma unroll
    for (int i = 0; i < 30; i++) g[i] = G[i];
}

__global__ void __launch_bounds__(128) k_gn_outflow(const double *__restrict__ xyz, const int32_t *__restrict__ conn,
                                                    int64_t ne, const double *__restrict__ u, ViscLaw L, GNOutflow of,
                                                    float *stage, int64_t e_begin, int64_t e_end) {
    const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= of.n) return;  // warp-uniform
    const int64_t e = of.elem[k];
    if (e < e_begin || e >= e_end) return;
    float Bi[9];
    const int32_t v0 = conn[e];
    geometry_fp64(xyz, v0, conn[ne + e], conn[2 * ne + e], conn[3 * ne + e], Bi);
    const double *x0 = xyz + 3 * (int64_t)v0;
    const double *f0 = xyz + 3 * (int64_t)of.face[3 * k], *f1 = xyz + 3 * (int64_t)of.face[3 * k + 1],
                 *f2 = xyz + 3 * (int64_t)of.face[3 * k + 2];
    // normal (f0 - f1) x (f0 - f2) and the area scaling |(f1 - f0) x (f2 - f0)|, FP64
    const double p1[3] = {f0[0] - f1[0], f0[1] - f1[1], f0[2] - f1[2]};
    const double p2[3] = {f0[0] - f2[0], f0[1] - f2[1], f0[2] - f2[2]};
    const double c[3] = {p1[1] * p2[2] - p1[2] * p2[1], p1[2] * p2[0] - p1[0] * p2[2], p1[0] * p2[1] - p1[1] * p2[0]};
    const double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    const float n[3] = {d2f_rn(c[0] / cn), d2f_rn(c[1] / cn), d2f_rn(c[2] / cn)};
    const float scale = d2f_rn(cn);  // |p1 x p2| = |(f1 - f0) x (f2 - f0)|
    float ue[30], un[10];
#pragma unroll
    for (int a = 0; a < 10; a++) {
        const double *up = u + 3 * (int64_t)conn[(int64_t)a * ne + e];
        ue[3 * a] = d2f_rn(up[0]);
        ue[3 * a + 1] = d2f_rn(up[1]);
        ue[3 * a + 2] = d2f_rn(up[2]);
        un[a] = ue[3 * a] * n[0] + ue[3 * a + 1] * n[1] + ue[3 * a + 2] * n[2];
    }
    constexpr double qa = 0.470142064105115, qb = 0.101286507323456;
    const double lam[7][3] = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0}, {1.0 - 2.0 * qa, qa, qa}, {qa, 1.0 - 2.0 * qa, qa},
                              {qa, qa, 1.0 - 2.0 * qa}, {1.0 - 2.0 * qb, qb, qb}, {qb, 1.0 - 2.0 * qb, qb},
                              {qb, qb, 1.0 - 2.0 * qb}};
    constexpr float wq[7] = {9.0f / 80.0f, 0.066197076394253f, 0.066197076394253f, 0.066197076394253f,
                             0.062969590272413f, 0.062969590272413f, 0.062969590272413f};
    // this lane's residual row r = (ri, rd) and matrix column (cj, ce), r = lane < 30
    const int r = lane < 30 ? lane : 29, ri = r / 3, rd = r - 3 * (r / 3);
    float res = 0.0f, col[30];
#pragma unroll
    for (int t = 0; t < 30; t++) col[t] = 0.0f;
#pragma unroll 1
    for (int q = 0; q < 7; q++) {
        float d[3];
#pragma unroll
        for (int t = 0; t < 3; t++)
            d[t] = d2f_rn(lam[q][0] * f0[t] + lam[q][1] * f1[t] + lam[q][2] * f2[t] - x0[t]);
        float xi[3];
#pragma unroll
        for (int t = 0; t < 3; t++) xi[t] = Bi[3 * t] * d[0] + Bi[3 * t + 1] * d[1] + Bi[3 * t + 2] * d[2];
        float phi[10], gr[30], g[30];
        p2_basis_at(xi[0], xi[1], xi[2], phi, gr);
        // physical gradients g_a,j = sum_c B^-1[c][j] ghat_a,c
#pragma unroll
        for (int a = 0; a < 10; a++)
#pragma unroll
            for (int j = 0; j < 3; j++)
                g[3 * a + j] = Bi[j] * gr[3 * a] + Bi[3 + j] * gr[3 * a + 1] + Bi[6 + j] * gr[3 * a + 2];
        float du[9], gn[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int t = 0; t < 9; t++) du[t] = 0.0f;
#pragma unroll
        for (int a = 0; a < 10; a++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
#pragma unroll
                for (int i = 0; i < 3; i++) du[3 * i + j] = fmaf(ue[3 * a + i], g[3 * a + j], du[3 * i + j]);
                gn[j] = fmaf(un[a], g[3 * a + j], gn[j]);
            }
        const float s01 = du[1] + du[3], s02 = du[2] + du[6], s12 = du[5] + du[7];
        const float gamma = sqrtf(2.0f * du[0] * du[0] + 2.0f * du[4] * du[4] + 2.0f * du[8] * du[8] + s01 * s01 +
                                  s02 * s02 + s12 * s12);
        const float cq = -scale * gn_eta(L, gamma) * wq[q];
        // residual row (ri, rd): cq phi_ri gn_rd; matrix column (cj, ce) = (ri, rd):
        // K[(i,d)][(cj,ce)] += cq phi_i g_cj,d n_ce
        float phr = 0.0f, gnr = 0.0f, gc[3] = {0.0f, 0.0f, 0.0f}, nce = 0.0f;
#pragma unroll
        for (int a = 0; a < 10; a++)
            if (a == ri) {
                phr = phi[a];
                gc[0] = g[3 * a];
                gc[1] = g[3 * a + 1];
                gc[2] = g[3 * a + 2];
            }
#pragma unroll
        for (int t = 0; t < 3; t++)
            if (t == rd) {
                gnr = gn[t];
                nce = n[t];
            }
        res = fmaf(cq * phr, gnr, res);
        if (of.matrix) {
            const float cn_ = cq * nce;
#pragma unroll
            for (int i = 0; i < 10; i++)
#pragma unroll
                for (int dd = 0; dd < 3; dd++) col[3 * i + dd] = fmaf(cn_ * phi[i], gc[dd], col[3 * i + dd]);
        }
    }
    if (lane < 30) {
        float *st = stage + e * kGNStride;
        st[kGNRes + lane] += res;
        if (of.matrix)
#pragma unroll
            for (int t = 0; t < 30; t++) st[32 * t + lane] += col[t];
    }
}

}  // namespace

void launch_gn_elem(const double *xyz, const int32_t *conn, int64_t ne, const double *u, const ViscLaw &law,
                    int newton, float *stage, int *d_err, cudaStream_t s, LaunchCounter &lc, int64_t e_begin,
                    int64_t e_end, const GNOutflow &outflow) {
    upload_gn_tables(s);
    if (e_end < 0) e_end = ne;
    if (e_end <= e_begin) return;
    k_gn_elem<<<(unsigned)ceil_div(e_end - e_begin, 32 * kGNWarps), 32 * kGNWarps, 0, s>>>(
        xyz, conn, ne, u, law, newton, stage, d_err, e_begin, e_end);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
    if (outflow.n > 0) {
        k_gn_outflow<<<(unsigned)ceil_div(outflow.n * 32, 128), 128, 0, s>>>(xyz, conn, ne, u, law, outflow, stage,
                                                                             e_begin, e_end);
        FEDD_CUDA(cudaGetLastError());
        lc.n++;
    }
}

void launch_gn_dense(const float *stage, int64_t first, int64_t count, double *Ke, double *re, cudaStream_t s,
                     double coeff_uu) {
    if (count == 0) return;
    k_gn_dense_add<<<(unsigned)ceil_div(count * 930, 256), 256, 0, s>>>(stage, first, count, Ke, re, coeff_uu);
    FEDD_CUDA(cudaGetLastError());
}

}  // namespace fedd
