// k_hyper.cu -- P2 elasticity / hyperelasticity: element stage (warp per
// element, FP32) and row stage (warp per node, deterministic gather).
//
// Element math follows the AceGen kernels FEDDLib calls for
// "LinearElasticity" (skr1, NeoHookQuadraticTets.f, 4-point rule code 18),
// "NonLinearElasticity" (skr2, NeoHookQuadraticTets2.f, 5-point rule code 19)
// and "NonLinearElasticity2" (skr3, NeoHookQuadraticTets3.f, code 19),
// restated from their strain energies (skr1: :27-32, 481-483; skr2: :28-30,
// 490-512; skr3: :25-31, 491-496) with FEDDLib's sign conventions
// (AssembleFE_LinElas_def.hpp:117-121, 167):
//     K = det B sum_q w_q G_a . A(F_q) . G_b,   r = -det B sum_q w_q P(F_q) G_a
// written for any law Psi(I1, J, I4a, I4b) through invariant derivatives:
//     K_(ai)(bj) = sum_kl psi_kl D_k[a,i] D_l[b,j] + d_ij (2 psi_1 G_a.G_b
//                  + sum_f 2 psi_4f (a_f.G_a)(a_f.G_b))
//                  + (psi_J / J) (c_a,i c_b,j - c_b,i c_a,j)
//     D_1 = 2 F G,  D_J = c = cof(F) G,  D_4f = 2 (F a_f)(a_f . G).
// Geometry (B, det B, cofactors) is computed in FP64, one thread per
// element; everything else is FP32.
#include <cuda_bf16.h>

#include "kernels.cuh"
#include "mlp_dev.cuh"

namespace fedd {
namespace {

constexpr int kWarps = 4;
__constant__ HyperTables c_htab;

// ---- laws ----------------------------------------------------------------
__device__ __forceinline__ void nh_matrix(int kind, float mu, float lam, float J, QPDerivs &d) {
    float iJ = 1.0f / J;
    d.d1[0] = 0.5f * mu;
    if (kind == kLawSKR2) {
        float lnJ = logf(J);
        d.d1[1] = (lam * lnJ - mu) * iJ;
        d.d2[4] = (mu + lam - lam * lnJ) * iJ * iJ;
    } else {  // skr1 (also the matrix of the fibre law and of the surrogate)
        d.d1[1] = -mu * iJ + 0.5f * lam * (J - iJ);
        d.d2[4] = mu * iJ * iJ + 0.5f * lam * (1.0f + iJ * iJ);
    }
}

__device__ __forceinline__ void fibre_terms(float k1, float k2, float I4, float &d1, float &d2) {
    float e = I4 - 1.0f;
    if (e > 0.0f) {
        float ex = expf(k2 * e * e);
        d1 = k1 * e * ex;
        d2 = k1 * ex * (1.0f + 2.0f * k2 * e * e);
    } else {
        d1 = 0.0f;
        d2 = 0.0f;
    }
}

// skr3, the isochoric split (NeoHookQuadraticTets3.f:25-31, 491-496, where
// v(208), v(214) and v(561) are the derivatives below with respect to
// I3 = J^2): Psi = mu/2 (J^-2/3 I1 - 3) + kappa/2 (J - 1)^2 with
// mu = E / (2 (1 + nu)), kappa = E / (3 (1 - 2 nu)).
__device__ __forceinline__ void skr3_terms(float mu, float kappa, float I1, float J, QPDerivs &d) {
    const float c = 1.0f / cbrtf(J);  // J^-1/3
    const float j23 = c * c, j53 = j23 / J, j83 = j53 * j23 * c;
    d.d1[0] = 0.5f * mu * j23;
    d.d1[1] = -(mu / 3.0f) * I1 * j53 + kappa * (J - 1.0f);
    d.d2[1] = -(mu / 3.0f) * j53;
    d.d2[4] = (5.0f * mu / 9.0f) * I1 * j83 + kappa;
}

// plain law at given invariants (used by the fused element stage, the
// plain-law QP kernel and the fallback of the surrogate)
__device__ __forceinline__ void law_plain(const LawParams &L, const float *inv, QPDerivs &d) {
#pragma unroll
    for (int k = 0; k < 4; k++) d.d1[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 10; k++) d.d2[k] = 0.0f;
    if (L.kind == kLawSKR3) {
        skr3_terms(L.mu, L.lam, inv[0], inv[1], d);
        return;
    }
    int kind = L.kind == kLawSKR2 ? kLawSKR2 : kLawSKR1;
    nh_matrix(kind, L.mu, L.lam, inv[1], d);
    if (L.kind == kLawAniso || L.kind == kLawMLP) {
        fibre_terms(L.k1, L.k2, inv[2], d.d1[2], d.d2[7]);
        fibre_terms(L.k1, L.k2, inv[3], d.d1[3], d.d2[9]);
    }
}

__device__ __forceinline__ float det3(const float *F) {
    return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) + F[2] * (F[3] * F[7] - F[4] * F[6]);
}

__device__ __forceinline__ void cof3(const float *F, float *C) {
    C[0] = F[4] * F[8] - F[5] * F[7];
    C[1] = F[5] * F[6] - F[3] * F[8];
    C[2] = F[3] * F[7] - F[4] * F[6];
    C[3] = F[2] * F[7] - F[1] * F[8];
    C[4] = F[0] * F[8] - F[2] * F[6];
    C[5] = F[1] * F[6] - F[0] * F[7];
    C[6] = F[1] * F[5] - F[2] * F[4];
    C[7] = F[2] * F[3] - F[0] * F[5];
    C[8] = F[0] * F[4] - F[1] * F[3];
}

// ---- element stage ----------------------------------------------------
// One warp per element, elements taken in batches of 32 per warp:
//   phase 1  FP64 geometry, one element of the batch per lane;
// then for each element of the batch:
//   phase Q  lane q < nq: F_q, cof F_q and the law's derivatives at F_q,
//            folded with the weight w_q det B into the scalars below;
//   phase V  one lane per (node a, point q): G = B^-T grad phi_a(q),
//            c = cof(F_q) G, f = F_q G, the fibre projections a_f . G and
//            node a's residual contribution at q;
//   phase K  one lane per 3 x 3 block (a, b), a <= b (55 blocks in two
//            passes), summing over q in registers
//              K_(ai)(bj) += gamma G_a.G_b d_ij + alpha c_ai c_bj
//                            - beta c_bi c_aj + (law-specific terms)
//            with gamma = 2 s psi_1, beta = s psi_J / J,
//            alpha = s (psi_JJ + psi_J / J), s = w_q det B;
//   epilogue both triangles into a shared-memory image of the element's
//            rows, then 16-byte coalesced stores.
// The pass of each block (c_pair_lane) is chosen so that within a pass the
// block stores and the transposed block stores into the image (row stride
// kSRow) put at most two lanes on one bank.
constexpr int kSRow = 44;  // floats per row of the shared element image
constexpr int kQS = 52;    // floats per quadrature-point record: 13 chunks of 16 B, so the records
                           // of q = 0..4 start in different bank groups
constexpr int kVS = 12;    // floats per (point, node) record: c0 c1 c2 G0 | G1 G2 f0 f1 | f2 g1 g2 -
// quadrature-point record: F 0-8, cof F 9-17, (gamma alpha beta kappa) 20,
// (phi1 phi2 chi1 chi2) 24, F a1 28, F a2 32, s psi_kl 36-45, residual
// scalars (-2 s psi_1, -s psi_J, -2 s psi_4a, -2 s psi_4b) 48
constexpr int kQScal = 20, kQFib = 24, kQFa1 = 28, kQFa2 = 32, kQHess = 36, kQRes = 48;
constexpr int kImage = 30 * kSRow;  // element image: 30 rows (column 30: the row's residual entry)
constexpr int kPhaseWords = 5 * kQS + 5 * 10 * kVS + 5 * 32;
static_assert(kPhaseWords <= kImage, "the phase buffers alias the element image");

// lane -> block (a << 4 | b) of pass 0 (entries 0-31) and pass 1 (32-54)
__constant__ uint8_t c_pair_lane[64] = {
    0x02, 0x03, 0x04, 0x05, 0x06, 0x08, 0x09, 0x13, 0x15, 0x17, 0x19, 0x23, 0x24, 0x28, 0x29, 0x33,
    0x38, 0x39, 0x44, 0x46, 0x49, 0x55, 0x56, 0x57, 0x59, 0x66, 0x68, 0x78, 0x79, 0x88, 0x89, 0x99,
    0x00, 0x01, 0x07, 0x11, 0x12, 0x14, 0x16, 0x18, 0x22, 0x25, 0x26, 0x27, 0x34, 0x35, 0x36, 0x37,
    0x45, 0x47, 0x48, 0x58, 0x67, 0x69, 0x77, 0xff, 0xff, 0xff, 0xff, 0xff, 0xff, 0xff, 0xff, 0xff};

// the scalars of one quadrature point that every block reads
template <int LAW>
struct PointScalars {
    float4 s;          // gamma alpha beta kappa
    float4 fib;        // phi1 phi2 chi1 chi2
    float fa1[3], fa2[3];
    float h[10];       // s psi_kl (surrogate)
    __device__ __forceinline__ void load(const float *Qq) {
        constexpr bool kFibre = (LAW == kLawAniso || LAW == kLawMLP || LAW == kLawMLPF);
        s = *reinterpret_cast<const float4 *>(Qq + kQScal);
        if (kFibre) {
            fib = *reinterpret_cast<const float4 *>(Qq + kQFib);
            const float4 x = *reinterpret_cast<const float4 *>(Qq + kQFa1);
            const float4 y = *reinterpret_cast<const float4 *>(Qq + kQFa2);
            fa1[0] = x.x; fa1[1] = x.y; fa1[2] = x.z;
            fa2[0] = y.x; fa2[1] = y.y; fa2[2] = y.z;
        }
        if (LAW == kLawMLP) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float4 z = *reinterpret_cast<const float4 *>(Qq + kQHess + 4 * k);
                if (4 * k < 10) h[4 * k] = z.x;
                if (4 * k + 1 < 10) h[4 * k + 1] = z.y;
                if (4 * k + 2 < 10) h[4 * k + 2] = z.z;
                if (4 * k + 3 < 10) h[4 * k + 3] = z.w;
            }
        }
    }
};

// one block (a, b) at one quadrature point: K += the block's integrand
template <int LAW>
__device__ __forceinline__ void block_update(float *K, const float *Va, const float *Vb, const PointScalars<LAW> &P) {
    constexpr bool kFibre = (LAW == kLawAniso || LAW == kLawMLP || LAW == kLawMLPF);
    constexpr bool kFullHess = (LAW == kLawMLP);
    constexpr bool kCross = (LAW == kLawSKR3);
    const float4 a0 = reinterpret_cast<const float4 *>(Va)[0], a1 = reinterpret_cast<const float4 *>(Va)[1];
    const float4 b0 = reinterpret_cast<const float4 *>(Vb)[0], b1 = reinterpret_cast<const float4 *>(Vb)[1];
    const float ca[3] = {a0.x, a0.y, a0.z}, cb[3] = {b0.x, b0.y, b0.z};
    float dg = P.s.x * (a0.w * b0.w + a1.x * b1.x + a1.y * b1.y);
    float t[3], n[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        t[j] = P.s.y * cb[j];
        n[j] = -P.s.z * ca[j];
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) K[3 * i + j] = fmaf(cb[i], n[j], fmaf(ca[i], t[j], K[3 * i + j]));
    if (kCross || kFibre) {
        const float4 a2 = reinterpret_cast<const float4 *>(Va)[2], b2 = reinterpret_cast<const float4 *>(Vb)[2];
        const float fa[3] = {a1.z, a1.w, a2.x}, fb[3] = {b1.z, b1.w, b2.x};
        if (kCross) {  // psi_1J (D_1 (x) D_J + D_J (x) D_1), D_1 = 2 f
            float kf[3], kc[3];
#pragma unroll
            for (int j = 0; j < 3; j++) {
                kf[j] = P.s.w * fb[j];
                kc[j] = P.s.w * cb[j];
            }
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) K[3 * i + j] = fmaf(fa[i], kc[j], fmaf(ca[i], kf[j], K[3 * i + j]));
        }
        if (kFibre) {
            const float g1 = a2.y * b2.y, g2 = a2.z * b2.z;
            dg = fmaf(P.fib.x, g1, fmaf(P.fib.y, g2, dg));
            if (!kFullHess) {  // psi_4f4f D_4f (x) D_4f, D_4f = 2 (a_f . G) F a_f
                const float x1 = P.fib.z * g1, x2 = P.fib.w * g2;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float y1 = x1 * P.fa1[i], y2 = x2 * P.fa2[i];
#pragma unroll
                    for (int j = 0; j < 3; j++) K[3 * i + j] = fmaf(y2, P.fa2[j], fmaf(y1, P.fa1[j], K[3 * i + j]));
                }
                if (LAW == kLawMLPF) {  // psi_4a4b (D_4a (x) D_4b + D_4b (x) D_4a), 4 s psi_4a4b in s.w
                    const float c12 = P.s.w * a2.y * b2.z, c21 = P.s.w * a2.z * b2.y;
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        const float y1 = c12 * P.fa1[i], y2 = c21 * P.fa2[i];
#pragma unroll
                        for (int j = 0; j < 3; j++) K[3 * i + j] = fmaf(y2, P.fa1[j], fmaf(y1, P.fa2[j], K[3 * i + j]));
                    }
                }
            } else {  // the full Hessian: sum_kl s psi_kl D_k[a] (x) D_l[b]
                float Da[4][3], Db[4][3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    Da[0][i] = 2.0f * fa[i];
                    Db[0][i] = 2.0f * fb[i];
                    Da[1][i] = ca[i];
                    Db[1][i] = cb[i];
                    Da[2][i] = 2.0f * a2.y * P.fa1[i];
                    Db[2][i] = 2.0f * b2.y * P.fa1[i];
                    Da[3][i] = 2.0f * a2.z * P.fa2[i];
                    Db[3][i] = 2.0f * b2.z * P.fa2[i];
                }
                const float *h = P.h;
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    const float E0 = h[0] * Db[0][j] + h[1] * Db[1][j] + h[2] * Db[2][j] + h[3] * Db[3][j];
                    const float E1 = h[1] * Db[0][j] + h[4] * Db[1][j] + h[5] * Db[2][j] + h[6] * Db[3][j];
                    const float E2 = h[2] * Db[0][j] + h[5] * Db[1][j] + h[7] * Db[2][j] + h[8] * Db[3][j];
                    const float E3 = h[3] * Db[0][j] + h[6] * Db[1][j] + h[8] * Db[2][j] + h[9] * Db[3][j];
#pragma unroll
                    for (int i = 0; i < 3; i++)
                        K[3 * i + j] += Da[0][i] * E0 + Da[1][i] * E1 + Da[2][i] * E2 + Da[3][i] * E3;
                }
            }
        }
    }
    K[0] += dg;
    K[4] += dg;
    K[8] += dg;
}

// LAW: kLawSKR1 / kLawSKR2 / kLawSKR3 / kLawAniso (fused plain law) or
// kLawMLP (reads per-QP derivatives of the surrogate network, adds the skr1
// matrix part).  Six CTAs per SM (at most 85 registers; the 33 KB of shared
// memory allow six) for every law but the full-Hessian surrogate, four for
// that one; without the bound the register allocation of these instances
// drifts between 72 and 160 with unrelated edits.
template <int LAW, bool HAS_U>
__global__ void __launch_bounds__(32 * kWarps, LAW == kLawMLP ? 4 : 6) k_hyper_elem(const double *__restrict__ xyz,
                                                            const int32_t *__restrict__ conn, int64_t ne,
                                                            const double *__restrict__ u, LawParams L,
                                                            const QPDerivs *__restrict__ qpd,
                                                            const uint8_t *__restrict__ qpfb, float *stage,
                                                            int want_res, int *err, int64_t e_begin, int64_t e_end) {
    constexpr bool kFibre = (LAW == kLawAniso || LAW == kLawMLP || LAW == kLawMLPF);
    __shared__ __align__(16) float sdphi[5][36];  // per point: grad_ref phi of the 10 nodes, zero padded
    __shared__ float sw[5];
    __shared__ float sBi[kWarps][32][11];
    __shared__ __align__(16) float sU[kWarps][2][36];  // nodal u of the element pair of phase Q
    __shared__ __align__(16) float sBuf[kWarps][kImage + 5 * kQS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nq = c_htab.nq;
    for (int i = threadIdx.x; i < 5 * 36; i += blockDim.x) {
        const int q = i / 36, k = i - 36 * q;
        (&sdphi[0][0])[i] = (q < nq && k < 30) ? (&c_htab.dphi[0][0][0])[30 * q + k] : 0.0f;
    }
    if (threadIdx.x < 5) sw[threadIdx.x] = (int)threadIdx.x < nq ? c_htab.w[threadIdx.x] : 0.0f;
    if (lane < 12) sU[w][lane / 6][30 + lane % 6] = 0.0f;
    __syncthreads();

    const unsigned p0 = c_pair_lane[lane], p1 = c_pair_lane[32 + lane];
    const int pa0 = (int)(p0 >> 4), pb0 = (int)(p0 & 15u);
    const bool two = p1 != 0xFFu;
    const int pa1 = two ? (int)(p1 >> 4) : 0, pb1 = two ? (int)(p1 & 15u) : 0;
    // per warp: point records of an even element (QA) | V | Rq, aliased by
    // the element image, then the point records of the odd element after it
    // (QB), which the even element's image leaves alone: phase Q runs once
    // per element pair, on 2 nq lanes
    float *QA = sBuf[w];            // [5][kQS]
    float *V = QA + 5 * kQS;        // [5][10][kVS]
    float *Rq = V + 5 * 10 * kVS;   // [5][32]: residual contribution of (node, component) at q
    float *QB = sBuf[w] + kImage;   // [5][kQS]
    float *O = sBuf[w];             // element image, aliases QA, V and Rq

    for (int64_t e0 = e_begin + ((int64_t)blockIdx.x * kWarps + w) * 32; e0 < e_end;
         e0 += (int64_t)gridDim.x * kWarps * 32) {
        {  // phase 1: FP64 geometry, one element per lane
            int64_t e = e0 + lane;
            if (e < e_end) {
                float Bi[9];
                float det = d2f_rn(geometry_fp64(xyz, conn[e], conn[ne + e], conn[2 * ne + e], conn[3 * ne + e], Bi));
#pragma unroll
                for (int k = 0; k < 9; k++) sBi[w][lane][k] = Bi[k];
                // det B, times the element's E_e / E when a modulus field is set (the
                // point weights w_q det B carry it into every block and residual term)
                sBi[w][lane][9] = L.escale ? det * L.escale[e] : det;
                if (!(det > 0.0f) && !(det < 0.0f)) set_dev_error(err, kDevBadDet);
            }
        }
        __syncwarp();
        const int nb = (int)min((int64_t)32, e_end - e0);
        for (int t = 0; t < nb; t++) {
            const int64_t el = e0 + t;
            float *Q = (t & 1) ? QB : QA;  // this element's point records
            float Bi[9];
#pragma unroll
            for (int k = 0; k < 9; k++) Bi[k] = sBi[w][t][k];
            // phase Q, at even t for the elements t and t + 1: one lane per
            // (element, quadrature point), lane = ep nq + q
            if ((t & 1) == 0) {
                if (HAS_U) {
                    for (int k = lane; k < 60; k += 32) {
                        const int ep = k >= 30 ? 1 : 0, kk = k - 30 * ep;
                        if (t + ep < nb) {
                            const int32_t node = conn[(int64_t)(kk / 3) * ne + el + ep];
                            sU[w][ep][kk] = d2f_rn(u[3 * (int64_t)node + kk % 3]);
                        }
                    }
                }
                __syncwarp();
                const int ep = lane >= nq ? 1 : 0, q = lane - ep * nq;
                if (lane < 2 * nq && t + ep < nb) {
                const float *Bq = sBi[w][t + ep];
                const float detB = Bq[9];
                float F[9];
                if (HAS_U) {
                    // H = sum_a u_a (x) grad_ref phi_a(q), nodes four at a time
                    float H[9];
#pragma unroll
                    for (int k = 0; k < 9; k++) H[k] = 0.0f;
                    const float4 *u4 = reinterpret_cast<const float4 *>(sU[w][ep]);
                    const float4 *d4 = reinterpret_cast<const float4 *>(sdphi[q]);
#pragma unroll
                    for (int g = 0; g < 3; g++) {
                        float uu[12], dd[12];
#pragma unroll
                        for (int m = 0; m < 3; m++) {
                            const float4 x = u4[3 * g + m], y = d4[3 * g + m];
                            uu[4 * m] = x.x; uu[4 * m + 1] = x.y; uu[4 * m + 2] = x.z; uu[4 * m + 3] = x.w;
                            dd[4 * m] = y.x; dd[4 * m + 1] = y.y; dd[4 * m + 2] = y.z; dd[4 * m + 3] = y.w;
                        }
#pragma unroll
                        for (int n = 0; n < 4; n++)
#pragma unroll
                            for (int i = 0; i < 3; i++)
#pragma unroll
                                for (int c = 0; c < 3; c++) H[3 * i + c] = fmaf(uu[3 * n + i], dd[3 * n + c], H[3 * i + c]);
                    }
                    // F = I + H B^-1
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int k = 0; k < 3; k++)
                            F[3 * i + k] = (i == k ? 1.0f : 0.0f) + H[3 * i] * Bq[k] + H[3 * i + 1] * Bq[3 + k] +
                                           H[3 * i + 2] * Bq[6 + k];
                } else {
#pragma unroll
                    for (int k = 0; k < 9; k++) F[k] = (k % 4 == 0) ? 1.0f : 0.0f;
                }
                float C[9];
                cof3(F, C);
                const float J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
                if (!(J > 0.0f)) set_dev_error(err, kDevBadDet);
                float Fa1[3] = {0.0f, 0.0f, 0.0f}, Fa2[3] = {0.0f, 0.0f, 0.0f}, inv[4];
                inv[0] = 0.0f;
#pragma unroll
                for (int k = 0; k < 9; k++) inv[0] = fmaf(F[k], F[k], inv[0]);
                inv[1] = J;
                inv[2] = inv[3] = 1.0f;
                if (kFibre) {
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        Fa1[i] = F[3 * i] * L.a1[0] + F[3 * i + 1] * L.a1[1] + F[3 * i + 2] * L.a1[2];
                        Fa2[i] = F[3 * i] * L.a2[0] + F[3 * i + 1] * L.a2[1] + F[3 * i + 2] * L.a2[2];
                    }
                    inv[2] = Fa1[0] * Fa1[0] + Fa1[1] * Fa1[1] + Fa1[2] * Fa1[2];
                    inv[3] = Fa2[0] * Fa2[0] + Fa2[1] * Fa2[1] + Fa2[2] * Fa2[2];
                }
                QPDerivs d;
                if (LAW == kLawMLP || LAW == kLawMLPF) {
                    const int64_t qi = (el + ep) * nq + q;
                    if (qpfb[qi]) {
                        law_plain(L, inv, d);
                    } else {
                        d = qpd[qi];
                        QPDerivs m;
#pragma unroll
                        for (int k = 0; k < 10; k++) m.d2[k] = 0.0f;
                        nh_matrix(kLawSKR1, L.mu, L.lam, J, m);
                        d.d1[0] += m.d1[0];
                        d.d1[1] += m.d1[1];
                        d.d2[4] += m.d2[4];
                    }
                } else {
                    law_plain(L, inv, d);
                }
                const float s = sw[q] * detB;
                const float psiJ_J = d.d1[1] / J;
                float *Qq = (ep ? QB : QA) + q * kQS;
#pragma unroll
                for (int k = 0; k < 9; k++) {
                    Qq[k] = F[k];
                    Qq[9 + k] = C[k];
                }
                const float beta = s * psiJ_J;
                const float alpha = LAW == kLawMLP ? beta : s * (d.d2[4] + psiJ_J);
                // the fourth scalar: 2 s psi_1J (skr3) or 4 s psi_4a4b (the fibre-block surrogate)
                *reinterpret_cast<float4 *>(Qq + kQScal) =
                    make_float4(2.0f * s * d.d1[0], alpha, beta, LAW == kLawMLPF ? 4.0f * s * d.d2[8] : 2.0f * s * d.d2[1]);
                *reinterpret_cast<float4 *>(Qq + kQRes) =
                    make_float4(-2.0f * s * d.d1[0], -s * d.d1[1], -2.0f * s * d.d1[2], -2.0f * s * d.d1[3]);
                if (kFibre) {
                    *reinterpret_cast<float4 *>(Qq + kQFib) =
                        make_float4(2.0f * s * d.d1[2], 2.0f * s * d.d1[3], 4.0f * s * d.d2[7], 4.0f * s * d.d2[9]);
                    *reinterpret_cast<float4 *>(Qq + kQFa1) = make_float4(Fa1[0], Fa1[1], Fa1[2], 0.0f);
                    *reinterpret_cast<float4 *>(Qq + kQFa2) = make_float4(Fa2[0], Fa2[1], Fa2[2], 0.0f);
                }
                if (LAW == kLawMLP) {
#pragma unroll
                    for (int k = 0; k < 10; k++) Qq[kQHess + k] = s * d.d2[k];
                }
                }
            }
            __syncwarp();
            // phase V: one lane per (point q, node a)
            for (int it = lane; it < 10 * nq; it += 32) {
                const int q = it / 10, a = it - 10 * q;
                const float *Qq = Q + q * kQS;
                const float g0 = sdphi[q][3 * a], g1 = sdphi[q][3 * a + 1], g2 = sdphi[q][3 * a + 2];
                float G[3];
#pragma unroll
                for (int k = 0; k < 3; k++) G[k] = Bi[k] * g0 + Bi[3 + k] * g1 + Bi[6 + k] * g2;
                float FC[20];
#pragma unroll
                for (int m = 0; m < 5; m++) {
                    const float4 x = reinterpret_cast<const float4 *>(Qq)[m];
                    FC[4 * m] = x.x; FC[4 * m + 1] = x.y; FC[4 * m + 2] = x.z; FC[4 * m + 3] = x.w;
                }
                float c[3], f[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    c[i] = FC[9 + 3 * i] * G[0] + FC[9 + 3 * i + 1] * G[1] + FC[9 + 3 * i + 2] * G[2];
                    f[i] = FC[3 * i] * G[0] + FC[3 * i + 1] * G[1] + FC[3 * i + 2] * G[2];
                }
                float ag1 = 0.0f, ag2 = 0.0f;
                if (kFibre) {
                    ag1 = L.a1[0] * G[0] + L.a1[1] * G[1] + L.a1[2] * G[2];
                    ag2 = L.a2[0] * G[0] + L.a2[1] * G[1] + L.a2[2] * G[2];
                }
                float4 *Vr = reinterpret_cast<float4 *>(V + (q * 10 + a) * kVS);
                Vr[0] = make_float4(c[0], c[1], c[2], G[0]);
                Vr[1] = make_float4(G[1], G[2], f[0], f[1]);
                Vr[2] = make_float4(f[2], ag1, ag2, 0.0f);
                if (want_res) {
                    const float4 rs = *reinterpret_cast<const float4 *>(Qq + kQRes);
                    float r[3];
#pragma unroll
                    for (int i = 0; i < 3; i++) r[i] = rs.x * f[i] + rs.y * c[i];
                    if (kFibre) {
                        const float4 x = *reinterpret_cast<const float4 *>(Qq + kQFa1);
                        const float4 y = *reinterpret_cast<const float4 *>(Qq + kQFa2);
                        const float h1 = rs.z * ag1, h2 = rs.w * ag2;
                        r[0] += h1 * x.x + h2 * y.x;
                        r[1] += h1 * x.y + h2 * y.y;
                        r[2] += h1 * x.z + h2 * y.z;
                    }
#pragma unroll
                    for (int i = 0; i < 3; i++) Rq[32 * q + 3 * a + i] = r[i];
                }
            }
            __syncwarp();
            // phase K: the blocks, summed over the points in registers
            float K0[9], K1[9];
#pragma unroll
            for (int k = 0; k < 9; k++) K0[k] = K1[k] = 0.0f;
            for (int q = 0; q < nq; q++) {
                PointScalars<LAW> P;
                P.load(Q + q * kQS);
                const float *Vq = V + q * 10 * kVS;
                block_update<LAW>(K0, Vq + pa0 * kVS, Vq + pb0 * kVS, P);
                if (two) block_update<LAW>(K1, Vq + pa1 * kVS, Vq + pb1 * kVS, P);
            }
            float r = 0.0f;
            if (want_res && lane < 30)
                for (int q = 0; q < nq; q++) r += Rq[32 * q + lane];
            __syncwarp();  // the phase buffers are dead: the element image overwrites them
#pragma unroll
            for (int pp = 0; pp < 2; pp++) {
                if (pp == 1 && !two) break;
                const int a = pp ? pa1 : pa0, b = pp ? pb1 : pb0;
                const float *Kb = pp ? K1 : K0;
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        O[kSRow * (3 * a + i) + 3 * b + j] = Kb[3 * i + j];
                        if (a != b) O[kSRow * (3 * b + j) + 3 * a + i] = Kb[3 * i + j];
                    }
            }
            if (lane < 30) O[kSRow * lane + kElemResCol] = r;  // row 3 a + i = lane
            __syncwarp();
            // global layout: rows of 32 floats, column 30 the residual entry, column 31 zero
            float4 *dst = reinterpret_cast<float4 *>(stage + el * kElemStride);
            for (int k = lane; k < kElemStride / 4; k += 32) {
                float4 v = *reinterpret_cast<const float4 *>(O + kSRow * (k >> 3) + 4 * (k & 7));
                if ((k & 7) == 7) v.w = 0.0f;
                dst[k] = v;
            }
            __syncwarp();
        }
        __syncwarp();
    }
}

// ---- row stage ----------------------------------------------------------
// One warp per node: walks the node's incidences in ascending element order,
// adds row a of each staged element matrix into shared-memory rows (FP32,
// one owner lane per value and incidence), then writes the node's three CSR
// rows once, converting to FP64.  The three values each lane needs from an
// incidence are streamed into a per-warp shared-memory ring with cp.async,
// kHRing - 1 incidences ahead of the arithmetic.
constexpr int kHRing = 4;
constexpr int kHStage = 100;  // floats per ring slot: three rows of 32 (values, residual entry, zero) | slot map 16 B
constexpr int kHSlots = 96;

// stage incidence t (of m) of a node into ring slot `slot` (a constant after
// unrolling): lanes 0-23 the three rows 3 a + i of the element matrix (row
// i = lane / 8, chunk lane % 8; column 30 of each row carries its residual
// entry), lane 24 the slot map; each lane's destination is ring slot + 4 lane.
// Every call commits one group, empty past the node's last incidence, so the
// wait counts hold.
__device__ __forceinline__ void hyper_stage(float *dst_lane, int slot, int t, int m, const IncList &il,
                                            const uint8_t *__restrict__ slots_node,
                                            const float *__restrict__ stage, int lane) {
    if (t < m) {  // warp-uniform: every lane takes part in the shuffle
        const uint32_t ea = incidence_at(il, t);
        const int a = (int)(ea & 15u);
        const float *Ke = stage + (size_t)(ea >> 4) * kElemStride;
        const void *src = lane < 24 ? static_cast<const void *>(Ke + 32 * (3 * a + (lane >> 3)) + 4 * (lane & 7))
                                    : static_cast<const void *>(slots_node + t * kSlotStride);
        if (lane < 25) cp_async16(dst_lane + slot * kHStage, src);
    }
    cp_async_commit();
}

// Accumulators: three planes (row components i) of stride 3 max_adj + 1, the
// last word of each a scratch word that lanes 30 and 31 write.
__global__ void __launch_bounds__(256) k_hyper_rows(const int64_t *__restrict__ inc_ptr,
                                                    const uint32_t *__restrict__ inc,
                                                    const uint8_t *__restrict__ slots,
                                                    const int64_t *__restrict__ adj_ptr,
                                                    const float *__restrict__ stage, const int64_t *__restrict__ rowptr,
                                                    double *vals, double *res, int64_t nnodes, int max_adj,
                                                    int64_t n_begin) {
    extern __shared__ __align__(16) float sacc[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int ps = 3 * max_adj + 1;
    float *ring = sacc + (size_t)w * (kHRing * kHStage + ((3 * ps + 3) & ~3));
    float *acc = ring + kHRing * kHStage;
    const bool lw = lane < 30;
    const int b = lw ? lane / 3 : 0, j = lw ? lane - 3 * (lane / 3) : 0;
    float *dst_lane = ring + 4 * lane;
    const uint8_t *pS = reinterpret_cast<const uint8_t *>(ring + kHSlots) + b;
    for (int64_t n = n_begin + (int64_t)blockIdx.x * nw + w; n < nnodes; n += (int64_t)gridDim.x * nw) {
        const int64_t i0 = inc_ptr[n], i1 = inc_ptr[n + 1];
        const int m = (int)(i1 - i0);
        const IncList il = load_incidences(inc, i0, m, lane);
        const uint8_t *slots_node = slots + i0 * kSlotStride;
#pragma unroll
        for (int t = 0; t < kHRing - 1; t++) hyper_stage(dst_lane, t, t, m, il, slots_node, stage, lane);
        const int K = (int)(adj_ptr[n + 1] - adj_ptr[n]);
        for (int c = lane; c < 3 * K; c += 32) acc[c] = acc[ps + c] = acc[2 * ps + c] = 0.0f;
        float r = 0.0f;
        for (int t0 = 0; t0 < m; t0 += kHRing) {
#pragma unroll
            for (int rs = 0; rs < kHRing; rs++) {
                const int t = t0 + rs;
                if (t >= m) break;
                cp_async_wait<kHRing - 2>();
                // the slot's copies are visible to the warp, and every lane is
                // done with the slot consumed in the previous step, refilled next
                __syncwarp();
                hyper_stage(dst_lane, (rs + kHRing - 1) % kHRing, t + kHRing - 1, m, il, slots_node, stage, lane);
                const float *S = ring + rs * kHStage;
                float *dst = acc + (lw ? 3 * pS[4 * rs * kHStage] + j : ps - 1);
                dst[0] += S[lane];
                dst[ps] += S[32 + lane];
                dst[2 * ps] += S[64 + lane];
                r += S[32 * (lane < 3 ? lane : 0) + kElemResCol];  // row i = lane's residual entry
            }
        }
        cp_async_wait<0>();
        __syncwarp();
        if (vals) {
            double *out = vals + rowptr[3 * n];
#pragma unroll
            for (int i = 0; i < 3; i++)
                for (int c = lane; c < 3 * K; c += 32) st_cs(out + i * 3 * K + c, f2d_exact(acc[i * ps + c]));
        }
        if (res && lane < 3) res[3 * n + lane] = f2d_exact(r);
        __syncwarp();
    }
}

// ---- surrogate path: invariants at every quadrature point ---------------
__global__ void k_hyper_invariants(const double *__restrict__ xyz, const int32_t *__restrict__ conn, int64_t ne,
                                   const double *__restrict__ u, LawParams L, float *inv, int *err, int64_t e_begin,
                                   int64_t e_end) {
    int64_t e = e_begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= e_end) return;
    float Bi[9];
    float det = d2f_rn(geometry_fp64(xyz, conn[e], conn[ne + e], conn[2 * ne + e], conn[3 * ne + e], Bi));
    (void)det;
    float ue[30];
#pragma unroll
    for (int a = 0; a < 10; a++) {
        int32_t node = conn[(int64_t)a * ne + e];
#pragma unroll
        for (int i = 0; i < 3; i++) ue[3 * a + i] = u ? d2f_rn(u[3 * (int64_t)node + i]) : 0.0f;
    }
    const int nq = c_htab.nq;
    for (int q = 0; q < nq; q++) {
        float Hr[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                float h = 0.0f;
#pragma unroll
                for (int a = 0; a < 10; a++) h = fmaf(ue[3 * a + i], c_htab.dphi[q][a][c], h);
                Hr[3 * i + c] = h;
            }
        float F[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int k = 0; k < 3; k++)
                F[3 * i + k] = (i == k ? 1.0f : 0.0f) + Hr[3 * i] * Bi[k] + Hr[3 * i + 1] * Bi[3 + k] +
                               Hr[3 * i + 2] * Bi[6 + k];
        float I1 = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; k++) I1 = fmaf(F[k], F[k], I1);
        float J = det3(F);
        if (!(J > 0.0f)) set_dev_error(err, kDevBadDet);
        float f1 = 0.0f, f2 = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float a1 = F[3 * i] * L.a1[0] + F[3 * i + 1] * L.a1[1] + F[3 * i + 2] * L.a1[2];
            float a2 = F[3 * i] * L.a2[0] + F[3 * i + 1] * L.a2[1] + F[3 * i + 2] * L.a2[2];
            f1 = fmaf(a1, a1, f1);
            f2 = fmaf(a2, a2, f2);
        }
        float4 v = make_float4(I1, J, f1, f2);
        reinterpret_cast<float4 *>(inv)[e * nq + q] = v;
    }
}

// plain law as a stand-alone QP kernel (same I/O as the surrogate kernel)
__global__ void k_law_qp_plain(LawParams L, const float *__restrict__ inv, int64_t nqp, QPDerivs *out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nqp) return;
    float4 v = reinterpret_cast<const float4 *>(inv)[i];
    float x[4] = {v.x, v.y, v.z, v.w};
    QPDerivs d;
    law_plain(L, x, d);
    out[i] = d;
}

__global__ void k_hyper_dense(const float *__restrict__ stage, int64_t first, int64_t count, double *Ke, double *re) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count * 930) return;
    int64_t e = t / 930;
    int k = (int)(t - e * 930);
    const float *S = stage + (first + e) * kElemStride;
    if (k < 900) {
        int p = k / 30, q = k % 30;
        Ke[e * 900 + k] = (double)S[32 * p + q];
    } else {
        re[e * 30 + (k - 900)] = (double)S[32 * (k - 900) + kElemResCol];
    }
}

}  // namespace

// ---- law evaluation for judging (FP32 math, one thread per F) -----------
__global__ void k_law_eval(LawParams L, MLPDev m, int use_mlp, int64_t n, const double *__restrict__ Fin,
                           double *psi_out, double *P, double *A) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    float F[9], C[9];
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = (float)Fin[9 * t + k];
    cof3(F, C);
    float J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
    float Fa[2][3], inv[4];
    inv[0] = 0.0f;
    for (int k = 0; k < 9; k++) inv[0] += F[k] * F[k];
    inv[1] = J;
    const float *af[2] = {L.a1, L.a2};
    for (int f = 0; f < 2; f++) {
        for (int i = 0; i < 3; i++) Fa[f][i] = F[3 * i] * af[f][0] + F[3 * i + 1] * af[f][1] + F[3 * i + 2] * af[f][2];
        inv[2 + f] = Fa[f][0] * Fa[f][0] + Fa[f][1] * Fa[f][1] + Fa[f][2] * Fa[f][2];
    }
    QPDerivs d;
    float psi = 0.0f;
    bool inside = true;
    if (use_mlp)
        for (int k = 0; k < 4; k++) inside = inside && inv[k] >= m.inv_lo[k] && inv[k] <= m.inv_hi[k];
    if (use_mlp && inside) {
        float x[4], y, g[4], h[16];
        float dk[4], d2k[4];
        for (int k = 0; k < 4; k++) x[k] = mlp_input(m, k, inv[k], dk[k], d2k[k]);
        mlp_eval_scalar(m, x, y, g, h);
        for (int k = 0; k < 10; k++) d.d2[k] = 0.0f;
        int kl = 0;
        for (int k = 0; k < 4; k++) {
            d.d1[k] = m.out_scale * g[k] * dk[k];
            for (int l = k; l < 4; l++, kl++)
                d.d2[kl] = m.out_scale * (h[4 * k + l] * dk[k] * dk[l] + (k == l ? g[k] * d2k[k] : 0.0f));
        }
        QPDerivs mm;
        for (int k = 0; k < 10; k++) mm.d2[k] = 0.0f;
        nh_matrix(kLawSKR1, L.mu, L.lam, J, mm);
        d.d1[0] += mm.d1[0];
        d.d1[1] += mm.d1[1];
        d.d2[4] += mm.d2[4];
        float lnJ = logf(J);
        psi = 0.5f * L.mu * (inv[0] - 3.0f) - L.mu * lnJ + 0.25f * L.lam * (J * J - 1.0f - 2.0f * lnJ) + m.out_scale * y;
    } else {
        law_plain(L, inv, d);
        float lnJ = logf(J);
        if (L.kind == kLawSKR2)
            psi = 0.5f * L.mu * (inv[0] - 3.0f) - L.mu * lnJ + 0.5f * L.lam * lnJ * lnJ;
        else if (L.kind == kLawSKR3)
            psi = 0.5f * L.mu * (inv[0] / (cbrtf(J) * cbrtf(J)) - 3.0f) + 0.5f * L.lam * (J - 1.0f) * (J - 1.0f);
        else
            psi = 0.5f * L.mu * (inv[0] - 3.0f) - L.mu * lnJ + 0.25f * L.lam * (J * J - 1.0f - 2.0f * lnJ);
        if (L.kind == kLawAniso || L.kind == kLawMLP)
            for (int f = 0; f < 2; f++) {
                float e = inv[2 + f] - 1.0f;
                if (e > 0.0f) psi += L.k1 / (2.0f * L.k2) * (expf(L.k2 * e * e) - 1.0f);
            }
    }
    psi_out[t] = psi;
    // P and A from the invariant form
    float D[4][9];
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) {
            D[0][3 * i + k] = 2.0f * F[3 * i + k];
            D[1][3 * i + k] = C[3 * i + k];
            D[2][3 * i + k] = 2.0f * Fa[0][i] * L.a1[k];
            D[3][3 * i + k] = 2.0f * Fa[1][i] * L.a2[k];
        }
    float H[4][4];
    {
        int kl = 0;
        for (int k = 0; k < 4; k++)
            for (int l = k; l < 4; l++, kl++) H[k][l] = H[l][k] = d.d2[kl];
    }
    for (int mm = 0; mm < 9; mm++) {
        float s = 0.0f;
        for (int k = 0; k < 4; k++) s += d.d1[k] * D[k][mm];
        P[9 * t + mm] = s;
    }
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
                for (int l = 0; l < 3; l++) {
                    float s = 0.0f;
                    for (int a = 0; a < 4; a++)
                        for (int b = 0; b < 4; b++) s += H[a][b] * D[a][3 * i + k] * D[b][3 * j + l];
                    if (i == j) s += 2.0f * d.d1[0] * (k == l) + 2.0f * d.d1[2] * L.a1[k] * L.a1[l] +
                                     2.0f * d.d1[3] * L.a2[k] * L.a2[l];
                    s += d.d1[1] * (C[3 * i + k] * C[3 * j + l] - C[3 * i + l] * C[3 * j + k]) / J;
                    A[81 * t + ((i * 3 + k) * 3 + j) * 3 + l] = s;
                }
}

// ---- launchers --------------------------------------------------------------
static void upload_htab(const HyperTables &tab, cudaStream_t s) {
    FEDD_CUDA(cudaMemcpyToSymbolAsync(c_htab, &tab, sizeof tab, 0, cudaMemcpyHostToDevice, s));
}

static int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

void launch_hyper_elem(const double *xyz, const int32_t *conn, int64_t ne, const double *u, const LawParams &law,
                       const HyperTables &tab, const QPDerivs *qpd, const uint8_t *qp_fallback, float *stage,
                       int want_res, int *d_err, cudaStream_t s, LaunchCounter &lc, int64_t e_begin,
                       int64_t e_end) {
    upload_htab(tab, s);
    if (e_end < 0) e_end = ne;
    int64_t warps = (e_end - e_begin + 31) / 32;
    unsigned grid = (unsigned)std::min<int64_t>((warps + kWarps - 1) / kWarps, (int64_t)sm_count() * 16);
    if (grid == 0) return;
    const bool hu = u != nullptr;
#define FEDD_HYPER(LAWK)                                                                                 \
    do {                                                                                                 \
        if (hu)                                                                                          \
            k_hyper_elem<LAWK, true><<<grid, 32 * kWarps, 0, s>>>(xyz, conn, ne, u, law, qpd, qp_fallback, \
                                                                  stage, want_res, d_err, e_begin, e_end); \
        else                                                                                             \
            k_hyper_elem<LAWK, false><<<grid, 32 * kWarps, 0, s>>>(xyz, conn, ne, u, law, qpd, qp_fallback, \
                                                                   stage, want_res, d_err, e_begin, e_end); \
    } while (0)
    switch (law.kind) {
    case kLawSKR2: FEDD_HYPER(kLawSKR2); break;
    case kLawSKR3: FEDD_HYPER(kLawSKR3); break;
    case kLawAniso: FEDD_HYPER(kLawAniso); break;
    case kLawMLP:
        if (law.mlp_fibre) FEDD_HYPER(kLawMLPF);
        else FEDD_HYPER(kLawMLP);
        break;
    default: FEDD_HYPER(kLawSKR1); break;
    }
#undef FEDD_HYPER
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

void launch_hyper_rows(const Graph &g, const float *stage, const int64_t *rowptr, double *vals, double *res,
                       int64_t nnodes, cudaStream_t s, LaunchCounter &lc, int64_t n_begin) {
    const int warps = 8;
    const int acc_words = (3 * (3 * g.max_adj + 1) + 3) & ~3;
    size_t smem = (size_t)warps * (kHRing * kHStage + acc_words) * sizeof(float);
    if (smem > 48 * 1024)
        FEDD_CUDA(cudaFuncSetAttribute(k_hyper_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    unsigned grid = (unsigned)std::min<int64_t>((nnodes - n_begin + warps - 1) / warps, (int64_t)sm_count() * 64);
    if (grid == 0) return;
    k_hyper_rows<<<grid, 32 * warps, smem, s>>>(g.inc_ptr.p, g.inc.p, g.slots.p, g.adj_ptr.p, stage, rowptr, vals,
                                                  res, nnodes, g.max_adj, n_begin);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}


void launch_hyper_invariants(const double *xyz, const int32_t *conn, int64_t ne, const double *u,
                             const LawParams &law, const HyperTables &tab, float *inv, int *d_err, cudaStream_t s,
                             LaunchCounter &lc, int64_t e_begin, int64_t e_end) {
    upload_htab(tab, s);
    if (e_end < 0) e_end = ne;
    if (e_end <= e_begin) return;
    k_hyper_invariants<<<ceil_div(e_end - e_begin, 128), 128, 0, s>>>(xyz, conn, ne, u, law, inv, d_err, e_begin,
                                                                        e_end);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

void launch_law_qp_plain(const LawParams &law, const float *inv, int64_t nqp, QPDerivs *out, cudaStream_t s,
                         LaunchCounter &lc) {
    if (nqp == 0) return;
    k_law_qp_plain<<<ceil_div(nqp, 256), 256, 0, s>>>(law, inv, nqp, out);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

void launch_law_eval(const LawParams &law, const MLPDev *m, int64_t n, const double *F, double *psi, double *P,
                     double *A, cudaStream_t s) {
    MLPDev mm{};
    if (m) mm = *m;
    if (n == 0) return;
    k_law_eval<<<ceil_div(n, 128), 128, 0, s>>>(law, mm, m != nullptr, n, F, psi, P, A);
    FEDD_CUDA(cudaGetLastError());
}

void launch_hyper_dense(const float *stage, int64_t first, int64_t count, double *Ke, double *re, cudaStream_t s) {
    if (count == 0) return;
    k_hyper_dense<<<ceil_div(count * 930, 256), 256, 0, s>>>(stage, first, count, Ke, re);
    FEDD_CUDA(cudaGetLastError());
}

}  // namespace fedd
