// mlp.cu -- MLP strain-energy surrogate: tensor-core inference with input
// derivatives at every quadrature point, and the training kernels.
//
// The network (no FEDDLib counterpart) maps normalised invariants
// x = (inv - shift) * scale, inv = (I1, J, I4a, I4b), to
//     net(x) = w3 . sp(W2 sp(W1 x + b1) + b2) + b3,   sp = softplus.
// The assembly needs dPsi/dinv and d2Psi/dinv2.  Forward-mode through the
// first layer gives 15 "channels" per point (h1, dh1/dx_k, d2h1/dx_kdx_l)
// that all meet the same second-layer weights, so the second layer is one
// GEMM of [points x 15 channels, H] by W2^T: it runs on the tensor cores
// (mma.sync m16n8k16, bf16 weights, activations split into bf16 hi + lo,
// FP32 accumulation).  Training (FP32, deterministic) minimises the Sobolev
// loss  mean( wpsi (y - t)^2 + wgrad |grad y - g|^2 )  with Adam.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <new>

#include "kernels.cuh"
#include "mlp_dev.cuh"

namespace fedd {
namespace {

constexpr int kH = 64;        // tensor-core path width
constexpr int kMlpWarps = 4;  // warps per CTA

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// bf16 hi part of (x, y) and the bf16 rounding of the remainders: x ~ hi + lo
// to about 16 significant bits
__device__ __forceinline__ void split_bf16(float x, float y, uint32_t &hi, uint32_t &lo) {
    const __nv_bfloat16 a = __float2bfloat16_rn(x), b = __float2bfloat16_rn(y);
    hi = pack_bf16(__bfloat162float(a), __bfloat162float(b));
    lo = pack_bf16(x - __bfloat162float(a), y - __bfloat162float(b));
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

struct MlpActive {
    int k[4];  // indices of the inputs with a non-zero normalisation scale, ascending
};

// Tensor-core surrogate derivatives, one warp per tile of 16 quadrature
// points (rows g and g + 8 of the m16n8k16 fragments for lane = 4 g + tq).
// With s1 = sigmoid(z1), t1 = s1 (1 - s1), D_k = W2 (s1 * W1[:, k]),
// s2 = sigmoid(z2), t2 = s2 (1 - s2):
//   dnet/dx_k      = sum_j w3_j s2_j D_kj
//   d2net/dx_k dx_l = sum_j w3_j t2_j D_kj D_lj + sum_i beta_i t1_i W1_ik W1_il,
//   beta = W2^T (w3 * s2)   (the backward product replaces the 10 forward
//                            second-derivative channels).
// Layer 2 runs on the tensor cores for the NA + 1 forward channels (h1 and
// s1 * W1[:, k] for the NA active inputs); its accumulators of n-tiles 2s and
// 2s + 1 are the A fragment of k-step s of the backward product, which is
// chained in registers.  Activations are split into bf16 hi + lo (weights are
// bf16), accumulation is FP32.  NTP n-tiles of layer 2 per pass keep the
// accumulators in registers (two passes recompute layer 1 when NA > 2).
template <int NA, int NTP>
__global__ void __launch_bounds__(32 * kMlpWarps, NA <= 2 ? 3 : 1) k_mlp_qp_tc(MLPDev m, MlpActive act, const float *__restrict__ inv,
                                                             int64_t nqp, QPDerivs *out, uint8_t *fb, int *fb_count) {
    constexpr int NC = 1 + NA, NH = NA * (NA + 1) / 2;
    __shared__ float sW1[kH][4], sb1[kH], sb2[kH], sw3[kH];
    __shared__ uint2 sB1[4][8][32], sB2[4][8][32];  // B fragments of W2 (layer 2) and W2^T (backward)
    __shared__ float sChain[kMlpWarps][16][2 * NA];  // the tile's input-map chain factors (dk, d2k)
    const __nv_bfloat16 *W1 = (const __nv_bfloat16 *)m.W1, *W2 = (const __nv_bfloat16 *)m.W2,
                        *w3 = (const __nv_bfloat16 *)m.w3;
    for (int t = threadIdx.x; t < kH; t += blockDim.x) {
        for (int k = 0; k < 4; k++) sW1[t][k] = __bfloat162float(W1[4 * t + k]);
        sb1[t] = m.b1[t];
        sb2[t] = m.b2[t];
        sw3[t] = __bfloat162float(w3[t]);
    }
    for (int t = threadIdx.x; t < 4 * 8 * 32; t += blockDim.x) {
        const int ks = t >> 8, nt = (t >> 5) & 7, ln = t & 31;
        const int n = 8 * nt + (ln >> 2), k0 = 16 * ks + 2 * (ln & 3);
        sB1[ks][nt][ln] = make_uint2(*reinterpret_cast<const uint32_t *>(W2 + (size_t)n * kH + k0),
                                     *reinterpret_cast<const uint32_t *>(W2 + (size_t)n * kH + k0 + 8));
        // W2^T: B(k = j, n = i) = W2[j][i]
        const __nv_bfloat16 *c = W2 + n;
        __nv_bfloat162 lo2, hi2;
        lo2.x = c[(size_t)k0 * kH];
        lo2.y = c[(size_t)(k0 + 1) * kH];
        hi2.x = c[(size_t)(k0 + 8) * kH];
        hi2.y = c[(size_t)(k0 + 9) * kH];
        sB2[ks][nt][ln] = make_uint2(*reinterpret_cast<uint32_t *>(&lo2), *reinterpret_cast<uint32_t *>(&hi2));
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, tq = lane & 3;
    const int64_t ntiles = (nqp + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * kMlpWarps + w; tile < ntiles; tile += (int64_t)gridDim.x * kMlpWarps) {
        const int64_t q0 = tile * 16 + g, q1 = q0 + 8;
        float x[2][4];
        bool in0 = q0 < nqp, in1 = q1 < nqp;
        {
            const float4 v0 = in0 ? reinterpret_cast<const float4 *>(inv)[q0] : make_float4(3.f, 1.f, 1.f, 1.f);
            const float4 v1 = in1 ? reinterpret_cast<const float4 *>(inv)[q1] : make_float4(3.f, 1.f, 1.f, 1.f);
            const float a0[4] = {v0.x, v0.y, v0.z, v0.w}, a1[4] = {v1.x, v1.y, v1.z, v1.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                in0 = in0 && a0[k] >= m.inv_lo[k] && a0[k] <= m.inv_hi[k];
                in1 = in1 && a1[k] >= m.inv_lo[k] && a1[k] <= m.inv_hi[k];
                float d0, d1, h0, h1;
                x[0][k] = mlp_input(m, k, a0[k], d0, h0);
                x[1][k] = mlp_input(m, k, a1[k], d1, h1);
#pragma unroll
                for (int a = 0; a < NA; a++)
                    if (tq == 0 && act.k[a] == k) {  // rows g and g + 8 of the tile
                        sChain[w][g][a] = d0;
                        sChain[w][g][NA + a] = h0;
                        sChain[w][g + 8][a] = d1;
                        sChain[w][g + 8][NA + a] = h1;
                    }
            }
        }
        float beta[8][4], G[2][NA], Hh[2][NH], t1s[4][4][2], pend[4];
#pragma unroll
        for (int t = 0; t < 8; t++) beta[t][0] = beta[t][1] = beta[t][2] = beta[t][3] = 0.0f;
#pragma unroll
        for (int r = 0; r < 2; r++) {
#pragma unroll
            for (int a = 0; a < NA; a++) G[r][a] = 0.0f;
#pragma unroll
            for (int a = 0; a < NH; a++) Hh[r][a] = 0.0f;
        }
#pragma unroll
        for (int p = 0; p < 8 / NTP; p++) {
            float acc[NC][NTP][4];
#pragma unroll
            for (int c = 0; c < NC; c++)
#pragma unroll
                for (int t = 0; t < NTP; t++) acc[c][t][0] = acc[c][t][1] = acc[c][t][2] = acc[c][t][3] = 0.0f;
#pragma unroll
            for (int ks = 0; ks < 4; ks++) {
                // layer 1 at this lane's (row, unit) positions of k-step ks
                float v[NC][4][2];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int i = 16 * ks + 2 * tq + (q & 1) + 8 * (q >> 1);
#pragma unroll
                    for (int r = 0; r < 2; r++) {
                        float z = sb1[i];
#pragma unroll
                        for (int k = 0; k < 4; k++) z = fmaf(sW1[i][k], x[r][k], z);
                        // softplus and sigmoid from one exponential, e = exp(-|z|) in
                        // (0, 1]: sp = max(z, 0) + log(1 + e), s = 1 / (1 + e) or e / (1 + e);
                        // fast-math log and reciprocal (a few ulp, below the bf16 hi + lo
                        // rounding of the layer-2 operand)
                        const float e1 = __expf(-fabsf(z)), r1 = __fdividef(1.0f, 1.0f + e1);
                        const float s1 = z >= 0.0f ? r1 : e1 * r1;
                        if (p == 0) t1s[ks][q][r] = s1 * (1.0f - s1);
                        v[0][q][r] = fmaxf(z, 0.0f) + __logf(1.0f + e1);
#pragma unroll
                        for (int a = 0; a < NA; a++) v[1 + a][q][r] = s1 * sW1[i][act.k[a]];
                    }
                }
                uint32_t Ahi[NC][4], Alo[NC][4];
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    split_bf16(v[c][0][0], v[c][1][0], Ahi[c][0], Alo[c][0]);
                    split_bf16(v[c][0][1], v[c][1][1], Ahi[c][1], Alo[c][1]);
                    split_bf16(v[c][2][0], v[c][3][0], Ahi[c][2], Alo[c][2]);
                    split_bf16(v[c][2][1], v[c][3][1], Ahi[c][3], Alo[c][3]);
                }
#pragma unroll
                for (int t = 0; t < NTP; t++) {
                    const uint2 B = sB1[ks][p * NTP + t][lane];
#pragma unroll
                    for (int c = 0; c < NC; c++) {
                        mma_bf16(acc[c][t], Ahi[c], B);
                        mma_bf16(acc[c][t], Alo[c], B);
                    }
                }
            }
            // layer-2 epilogue; every two n-tiles feed one k-step of the backward product
#pragma unroll
            for (int t = 0; t < NTP; t++) {
                const int nt = p * NTP + t;
                float vv[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int r = e >> 1, j = 8 * nt + 2 * tq + (e & 1);
                    // sigmoid with a fast reciprocal (a few ulp, below the bf16
                    // hi + lo rounding of the backward product's operand)
                    const float z2 = acc[0][t][e] + sb2[j];
                    const float e2 = __expf(-fabsf(z2)), r2 = __fdividef(1.0f, 1.0f + e2);
                    const float s2 = z2 >= 0.0f ? r2 : e2 * r2;
                    const float t2 = s2 * (1.0f - s2), cw = sw3[j];
                    int ab = 0;
#pragma unroll
                    for (int a = 0; a < NA; a++) {
                        const float Da = acc[1 + a][t][e];
                        G[r][a] = fmaf(cw * s2, Da, G[r][a]);
#pragma unroll
                        for (int b = a; b < NA; b++, ab++) Hh[r][ab] = fmaf(cw * t2 * Da, acc[1 + b][t][e], Hh[r][ab]);
                    }
                    vv[e] = cw * s2;
                }
                if ((nt & 1) == 0) {
#pragma unroll
                    for (int e = 0; e < 4; e++) pend[e] = vv[e];
                } else {
                    uint32_t Ahi[4], Alo[4];
                    split_bf16(pend[0], pend[1], Ahi[0], Alo[0]);
                    split_bf16(pend[2], pend[3], Ahi[1], Alo[1]);
                    split_bf16(vv[0], vv[1], Ahi[2], Alo[2]);
                    split_bf16(vv[2], vv[3], Ahi[3], Alo[3]);
                    const int ks2 = nt >> 1;
#pragma unroll
                    for (int t2i = 0; t2i < 8; t2i++) {
                        const uint2 B = sB2[ks2][t2i][lane];
                        mma_bf16(beta[t2i], Ahi, B);
                        mma_bf16(beta[t2i], Alo, B);
                    }
                }
            }
        }
        // sum_i beta_i t1_i W1_ik W1_il over this lane's hidden units
#pragma unroll
        for (int ks = 0; ks < 4; ks++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int i = 16 * ks + 2 * tq + (q & 1) + 8 * (q >> 1);
                float wk[NA];
#pragma unroll
                for (int a = 0; a < NA; a++) wk[a] = sW1[i][act.k[a]];
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    const float bt = beta[2 * ks + (q >> 1)][2 * r + (q & 1)] * t1s[ks][q][r];
                    int ab = 0;
#pragma unroll
                    for (int a = 0; a < NA; a++)
#pragma unroll
                        for (int b = a; b < NA; b++, ab++) Hh[r][ab] = fmaf(bt * wk[a], wk[b], Hh[r][ab]);
                }
            }
        // reduce over the four lanes of each row
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
            for (int o = 1; o <= 2; o <<= 1) {
#pragma unroll
                for (int a = 0; a < NA; a++) G[r][a] += __shfl_xor_sync(0xffffffffu, G[r][a], o);
#pragma unroll
                for (int a = 0; a < NH; a++) Hh[r][a] += __shfl_xor_sync(0xffffffffu, Hh[r][a], o);
            }
        if (tq == 0) {
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int64_t q = r ? q1 : q0;
                if (q >= nqp) continue;
                const bool inside = r ? in1 : in0;
                // the chain factors dx_k / dinv_k and d2x_k / dinv_k2 of the input
                // map, for the active inputs k = act.k[a] (stored at the tile's start)
                float dk[NA], d2k[NA];
#pragma unroll
                for (int a = 0; a < NA; a++) {
                    dk[a] = sChain[w][g + 8 * r][a];
                    d2k[a] = sChain[w][g + 8 * r][NA + a];
                }
                QPDerivs d;
#pragma unroll
                for (int k = 0; k < 4; k++) d.d1[k] = 0.0f;
#pragma unroll
                for (int k = 0; k < 10; k++) d.d2[k] = 0.0f;
                int ab = 0;
#pragma unroll
                for (int a = 0; a < NA; a++) {
                    const int k = act.k[a];
                    d.d1[k] = m.out_scale * G[r][a] * dk[a];
#pragma unroll
                    for (int b = a; b < NA; b++, ab++) {
                        const int l = act.k[b];
                        // packed symmetric index of (k, l), k <= l: 00,01,02,03,11,12,13,22,23,33
                        const int kl = k * 4 - k * (k - 1) / 2 + (l - k);
                        d.d2[kl] = m.out_scale * (Hh[r][ab] * dk[a] * dk[b] + (a == b ? G[r][a] * d2k[a] : 0.0f));
                    }
                }
                out[q] = d;
                fb[q] = inside ? 0 : 1;
                if (!inside) atomicAdd(fb_count, 1);
            }
        }
    }
}

// general width: one thread per point (CUDA cores)
__global__ void k_mlp_qp_scalar(MLPDev m, const float *__restrict__ inv, int64_t nqp, QPDerivs *out, uint8_t *fb,
                                int *fb_count) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= nqp) return;
    float4 v = reinterpret_cast<const float4 *>(inv)[q];
    float a[4] = {v.x, v.y, v.z, v.w}, x[4], dk[4], d2k[4];
    bool inside = true;
    for (int k = 0; k < 4; k++) {
        inside = inside && a[k] >= m.inv_lo[k] && a[k] <= m.inv_hi[k];
        x[k] = mlp_input(m, k, a[k], dk[k], d2k[k]);
    }
    float y, g[4], h[16];
    mlp_eval_scalar(m, x, y, g, h);
    QPDerivs d;
    int kl = 0;
    for (int k = 0; k < 4; k++) {
        d.d1[k] = m.out_scale * g[k] * dk[k];
        for (int l = k; l < 4; l++, kl++)
            d.d2[kl] = m.out_scale * (h[4 * k + l] * dk[k] * dk[l] + (k == l ? g[k] * d2k[k] : 0.0f));
    }
    out[q] = d;
    fb[q] = inside ? 0 : 1;
    if (!inside) atomicAdd(fb_count, 1);
}

int sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

void launch_mlp_qp(const MLPDev &m, const LawParams &law, const float *inv, int64_t nqp, QPDerivs *out,
                   uint8_t *fallback, int *d_count, cudaStream_t s, LaunchCounter &lc) {
    (void)law;
    if (nqp == 0) return;
    MlpActive act{};
    int na = 0;
    for (int k = 0; k < 4; k++)
        if (m.in_scale[k] != 0.0f) act.k[na++] = k;
    if (m.hidden == kH && na > 0) {
        const int64_t ntiles = (nqp + 15) / 16;
        const unsigned grid = (unsigned)std::min<int64_t>((ntiles + kMlpWarps - 1) / kMlpWarps, (int64_t)sms() * 16);
        switch (na) {
        case 1: k_mlp_qp_tc<1, 8><<<grid, 32 * kMlpWarps, 0, s>>>(m, act, inv, nqp, out, fallback, d_count); break;
        case 2: k_mlp_qp_tc<2, 8><<<grid, 32 * kMlpWarps, 0, s>>>(m, act, inv, nqp, out, fallback, d_count); break;
        case 3: k_mlp_qp_tc<3, 2><<<grid, 32 * kMlpWarps, 0, s>>>(m, act, inv, nqp, out, fallback, d_count); break;
        default: k_mlp_qp_tc<4, 2><<<grid, 32 * kMlpWarps, 0, s>>>(m, act, inv, nqp, out, fallback, d_count); break;
        }
    } else {
        k_mlp_qp_scalar<<<ceil_div(nqp, 128), 128, 0, s>>>(m, inv, nqp, out, fallback, d_count);
    }
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

// ============================ training =====================================
namespace {

// C[M x N] = sum_k A(m,k) B(k,n), FP32, 64x64 tiles, 256 threads (4x4 each).
// TA: A stored K x M (A(m,k) = A[k*lda + m]) else M x K.
// TB: B stored N x K (B(k,n) = B[n*ldb + k]) else K x N.
// Split-K: blockIdx.z handles K range [z*kc, (z+1)*kc), writes C + z*M*N.
template <bool TA, bool TB>
__global__ void k_sgemm(const float *__restrict__ A, const float *__restrict__ B, float *C, int M, int N, int64_t K,
                        int64_t kc) {
    __shared__ float As[16][65], Bs[16][65];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int64_t k_begin = (int64_t)blockIdx.z * kc, k_end = std::min<int64_t>(K, k_begin + kc);
    float acc[4][4] = {{0}};
    for (int64_t k0 = k_begin; k0 < k_end; k0 += 16) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            const int kk = t / 64, mm = t % 64;
            const int64_t k = k0 + kk;
            float av = 0.0f, bv = 0.0f;
            if (k < k_end) {
                const int gm = m0 + mm, gn = n0 + mm;
                if (gm < M) av = TA ? A[k * M + gm] : A[(int64_t)gm * K + k];
                if (gn < N) bv = TB ? B[(int64_t)gn * K + k] : B[k * N + gn];
            }
            As[kk][mm] = av;
            Bs[kk][mm] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++)
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(As[kk][ty * 4 + i], Bs[kk][tx * 4 + j], acc[i][j]);
        __syncthreads();
    }
    float *Cz = C + (int64_t)blockIdx.z * M * N;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
            if (gm < M && gn < N) Cz[(int64_t)gm * N + gn] = acc[i][j];
        }
}

// out[c] = sum over rows r (fixed order) of in[r * cols + c]
__global__ void k_colsum(const float *__restrict__ in, int64_t rows, int cols, float *out) {
    __shared__ float red[256];
    const int c = blockIdx.x;
    float s = 0.0f;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) s += in[r * cols + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

struct TrainParams {
    const float *W1, *b1, *W2, *b2, *w3;
    float b3;
};

// forward layer 1: X1 = [H1; DH1_0..3] (5B x H), caches S1, T1
__global__ void k_tr_l1(TrainParams P, int H, const float *__restrict__ X, const int64_t *__restrict__ idx, int64_t B,
                        float *X1, float *S1, float *T1) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= B * H) return;
    const int64_t s = t / H;
    const int i = (int)(t - s * H);
    const float *x = X + 4 * idx[s];
    float z = P.b1[i];
    for (int k = 0; k < 4; k++) z = fmaf(P.W1[4 * i + k], x[k], z);
    const float sg = 1.0f / (1.0f + expf(-z)), tg = sg * (1.0f - sg);
    const float hv = z > 20.0f ? z : log1pf(expf(z));
    X1[s * H + i] = hv;
    for (int k = 0; k < 4; k++) X1[((1 + k) * B + s) * H + i] = sg * P.W1[4 * i + k];
    S1[s * H + i] = sg;
    T1[s * H + i] = tg;
}

// forward layer 2 + loss + start of the backward pass, one warp per sample
__global__ void k_tr_l2(TrainParams P, int H, const float *__restrict__ Z2, const float *__restrict__ ty,
                        const float *__restrict__ tgr, const int64_t *__restrict__ idx, int64_t B, float wpsi,
                        float wgrad, float *D, float *GW3, float *lossv, float *ey_out) {
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B) return;
    float yp = 0.0f, gp[4] = {0, 0, 0, 0};
    for (int j = lane; j < H; j += 32) {
        const float z = Z2[s * H + j] + P.b2[j];
        const float sg = 1.0f / (1.0f + expf(-z));
        yp = fmaf(P.w3[j], z > 20.0f ? z : log1pf(expf(z)), yp);
        for (int k = 0; k < 4; k++) gp[k] = fmaf(P.w3[j] * sg, Z2[((1 + k) * B + s) * H + j], gp[k]);
    }
    const float y = warp_sum(yp) + P.b3;
    float g[4];
    for (int k = 0; k < 4; k++) g[k] = warp_sum(gp[k]);
    const int64_t si = idx[s];
    const float ey = 2.0f * wpsi * (y - ty[si]);
    float eg[4], l = wpsi * (y - ty[si]) * (y - ty[si]);
    for (int k = 0; k < 4; k++) {
        const float dk = g[k] - tgr[4 * si + k];
        eg[k] = 2.0f * wgrad * dk;
        l += wgrad * dk * dk;
    }
    for (int j = lane; j < H; j += 32) {
        const float z = Z2[s * H + j] + P.b2[j];
        const float sg = 1.0f / (1.0f + expf(-z)), tg = sg * (1.0f - sg);
        const float hv = z > 20.0f ? z : log1pf(expf(z));
        float dz2 = ey * P.w3[j] * sg, gw = ey * hv;
        for (int k = 0; k < 4; k++) {
            const float dzk = Z2[((1 + k) * B + s) * H + j];
            dz2 = fmaf(eg[k] * P.w3[j] * tg, dzk, dz2);
            gw = fmaf(eg[k] * sg, dzk, gw);
            D[((1 + k) * B + s) * H + j] = eg[k] * P.w3[j] * sg;
        }
        D[s * H + j] = dz2;
        GW3[s * H + j] = gw;
    }
    if (lane == 0) {
        lossv[s] = l;
        ey_out[s] = ey;
    }
}

// backward through layer 1: per-sample contributions to gW1 and gb1
__global__ void k_tr_l1b(TrainParams P, int H, const float *__restrict__ X, const int64_t *__restrict__ idx, int64_t B,
                         const float *__restrict__ DX1, const float *__restrict__ S1, const float *__restrict__ T1,
                         float *G1) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= B * H) return;
    const int64_t s = t / H;
    const int i = (int)(t - s * H);
    const float *x = X + 4 * idx[s];
    const float sg = S1[s * H + i], tg = T1[s * H + i];
    float dz = DX1[s * H + i] * sg;
    float dd[4];
    for (int k = 0; k < 4; k++) {
        dd[k] = DX1[((1 + k) * B + s) * H + i];
        dz = fmaf(dd[k] * tg, P.W1[4 * i + k], dz);
    }
    // layout per sample: [gW1 (H x 4) | gb1 (H)]
    float *o = G1 + s * (5 * H);
    for (int k = 0; k < 4; k++) o[4 * i + k] = dd[k] * sg + dz * x[k];
    o[4 * H + i] = dz;
}

__global__ void k_adam(float *p, const float *g, float *m1, float *m2, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, float scale) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * scale;
    m1[i] = b1 * m1[i] + (1.0f - b1) * gi;
    m2[i] = b2 * m2[i] + (1.0f - b2) * gi * gi;
    p[i] -= lr * (m1[i] / c1) / (sqrtf(m2[i] / c2) + eps);
}

}  // namespace
}  // namespace fedd

using namespace fedd;

struct fedd_trainer {
    int device = 0, H = 64;
    int64_t n = 0;
    DBuf<float> X, ty, tg;
    // parameters (flat): W1 (4H) | b1 (H) | W2 (HH) | b2 (H) | w3 (H) | b3 (1)
    DBuf<float> par, grad, m1, m2;
    int64_t step = 0;
    // workspace for a batch
    int64_t B = 0;
    DBuf<int64_t> idx;
    DBuf<float> X1, S1, T1, Z2, D, DX1, GW3, G1, lossv, ey, part;
    DBuf<float> lsum;  // the batch's summed loss (one float, allocated once)
    std::vector<int64_t> perm;
    uint64_t rng = 0;
    int64_t cursor = 0;
    std::string err;
    int nparams() const { return 4 * H + H + H * H + H + H + 1; }
    TrainParams tp() const {
        TrainParams t;
        t.W1 = par.p;
        t.b1 = par.p + 4 * H;
        t.W2 = par.p + 5 * H;
        t.b2 = par.p + 5 * H + H * H;
        t.w3 = par.p + 6 * H + H * H;
        t.b3 = 0.0f;
        return t;
    }
};

namespace {

void tr_workspace(fedd_trainer *t, int64_t B) {
    if (t->B == B) return;
    const int H = t->H;
    t->B = B;
    t->idx.alloc(B);
    t->X1.alloc(5 * B * H);
    t->S1.alloc(B * H);
    t->T1.alloc(B * H);
    t->Z2.alloc(5 * B * H);
    t->D.alloc(5 * B * H);
    t->DX1.alloc(5 * B * H);
    t->GW3.alloc(B * H);
    t->G1.alloc(B * 5 * H);
    t->lossv.alloc(B);
    t->ey.alloc(B);
}

// loss and gradient (sum over the batch, not yet divided by B) into t->grad
float tr_forward_backward(fedd_trainer *t, int64_t B, float wpsi, float wgrad, float b3) {
    const int H = t->H;
    cudaStream_t s = 0;
    TrainParams P = t->tp();
    P.b3 = b3;
    k_tr_l1<<<ceil_div(B * H, 256), 256, 0, s>>>(P, H, t->X.p, t->idx.p, B, t->X1.p, t->S1.p, t->T1.p);
    {  // Z2 (5B x H) = X1 (5B x H) . W2^T
        dim3 grid(ceil_div(H, 64), ceil_div(5 * B, 64), 1);
        k_sgemm<false, true><<<grid, 256, 0, s>>>(t->X1.p, P.W2, t->Z2.p, (int)(5 * B), H, H, H);
    }
    k_tr_l2<<<ceil_div(B * 32, 256), 256, 0, s>>>(P, H, t->Z2.p, t->ty.p, t->tg.p, t->idx.p, B, wpsi, wgrad, t->D.p,
                                                  t->GW3.p, t->lossv.p, t->ey.p);
    float *g = t->grad.p;
    // gradient layout: W1 (4 H) | b1 (H) | W2 (H H) | b2 (H) | w3 (H) | b3; b1's
    // part is written together with W1's (one column sum over 5 H columns)
    float *gW1 = g, *gW2 = g + 5 * H, *gb2 = g + 5 * H + H * H, *gw3 = g + 6 * H + H * H,
          *gb3 = g + 7 * H + H * H;
    {  // gW2 (H x H) = D^T (H x 5B) . X1 (5B x H), split-K then fixed-order sum
        const int64_t K = 5 * B;
        const int64_t nz = std::min<int64_t>(256, (K + 4095) / 4096);
        const int64_t kc = ((K + nz - 1) / nz + 15) / 16 * 16;
        const int64_t zc = (K + kc - 1) / kc;
        if (t->part.n < (size_t)(zc * H * H)) t->part.alloc(zc * H * H);
        dim3 grid(ceil_div(H, 64), ceil_div(H, 64), (unsigned)zc);
        k_sgemm<true, false><<<grid, 256, 0, s>>>(t->D.p, t->X1.p, t->part.p, H, H, K, kc);
        k_colsum<<<H * H, 256, 0, s>>>(t->part.p, zc, H * H, gW2);
    }
    {  // DX1 (5B x H) = D (5B x H) . W2 (H x H)
        dim3 grid(ceil_div(H, 64), ceil_div(5 * B, 64), 1);
        k_sgemm<false, false><<<grid, 256, 0, s>>>(t->D.p, P.W2, t->DX1.p, (int)(5 * B), H, H, H);
    }
    k_tr_l1b<<<ceil_div(B * H, 256), 256, 0, s>>>(P, H, t->X.p, t->idx.p, B, t->DX1.p, t->S1.p, t->T1.p, t->G1.p);
    k_colsum<<<5 * H, 256, 0, s>>>(t->G1.p, B, 5 * H, gW1);  // gW1 | gb1 contiguous
    k_colsum<<<H, 256, 0, s>>>(t->D.p, B, H, gb2);
    k_colsum<<<H, 256, 0, s>>>(t->GW3.p, B, H, gw3);
    k_colsum<<<1, 256, 0, s>>>(t->ey.p, B, 1, gb3);
    FEDD_CUDA(cudaGetLastError());
    if (!t->lsum.p) t->lsum.alloc(1);
    k_colsum<<<1, 256, 0, s>>>(t->lossv.p, B, 1, t->lsum.p);
    float L = 0;
    FEDD_CUDA(cudaMemcpyAsync(&L, t->lsum.p, sizeof L, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    return L;
}

template <class F> fedd_status tguard(fedd_trainer *t, F &&f) {
    try {
        f();
        return FEDD_OK;
    } catch (const Status &s) {
        if (t) t->err = s.msg;
        return s.code;
    } catch (const CudaError &e) {
        if (t) t->err = std::string(e.what) + ": " + cudaGetErrorString(e.code);
        return FEDD_ERR_CUDA;
    } catch (...) {
        return FEDD_ERR_CUDA;
    }
}

uint64_t sm64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" {

fedd_status fedd_trainer_create(int32_t hidden, int64_t n, const float *x, const float *tpsi, const float *tgrad,
                                int device, fedd_trainer **out) {
    if (!out || hidden < 4 || hidden > 512 || n <= 0 || !x || !tpsi || !tgrad) return FEDD_ERR_ARG;
    fedd_trainer *t = new (std::nothrow) fedd_trainer;
    if (!t) return FEDD_ERR_NOMEM;
    fedd_status st = tguard(t, [&] {
        FEDD_CUDA(cudaSetDevice(device));
        t->device = device;
        t->H = hidden;
        t->n = n;
        t->X.upload(x, n * 4);
        t->ty.upload(tpsi, n);
        t->tg.upload(tgrad, n * 4);
        const int np = t->nparams();
        t->par.alloc(np);
        t->grad.alloc(np);
        t->m1.alloc(np);
        t->m2.alloc(np);
        t->par.zero();
        t->m1.zero();
        t->m2.zero();
        FEDD_CUDA(cudaDeviceSynchronize());
    });
    if (st != FEDD_OK) {
        delete t;
        return st;
    }
    *out = t;
    return FEDD_OK;
}

fedd_status fedd_trainer_set_params(fedd_trainer *t, const float *W1, const float *b1, const float *W2,
                                    const float *b2, const float *w3, float b3) {
    if (!t || !W1 || !b1 || !W2 || !b2 || !w3) return FEDD_ERR_ARG;
    return tguard(t, [&] {
        FEDD_CUDA(cudaSetDevice(t->device));
        const int H = t->H;
        std::vector<float> h(t->nparams());
        std::memcpy(h.data(), W1, 4 * H * sizeof(float));
        std::memcpy(h.data() + 4 * H, b1, H * sizeof(float));
        std::memcpy(h.data() + 5 * H, W2, (size_t)H * H * sizeof(float));
        std::memcpy(h.data() + 5 * H + H * H, b2, H * sizeof(float));
        std::memcpy(h.data() + 6 * H + H * H, w3, H * sizeof(float));
        h[7 * H + H * H] = b3;
        FEDD_CUDA(cudaMemcpy(t->par.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
        t->m1.zero();
        t->m2.zero();
        t->step = 0;
        FEDD_CUDA(cudaDeviceSynchronize());
    });
}

fedd_status fedd_trainer_get_params(fedd_trainer *t, float *W1, float *b1, float *W2, float *b2, float *w3, float *b3) {
    if (!t || !W1 || !b1 || !W2 || !b2 || !w3 || !b3) return FEDD_ERR_ARG;
    return tguard(t, [&] {
        FEDD_CUDA(cudaSetDevice(t->device));
        const int H = t->H;
        std::vector<float> h(t->nparams());
        FEDD_CUDA(cudaMemcpy(h.data(), t->par.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
        std::memcpy(W1, h.data(), 4 * H * sizeof(float));
        std::memcpy(b1, h.data() + 4 * H, H * sizeof(float));
        std::memcpy(W2, h.data() + 5 * H, (size_t)H * H * sizeof(float));
        std::memcpy(b2, h.data() + 5 * H + H * H, H * sizeof(float));
        std::memcpy(w3, h.data() + 6 * H + H * H, H * sizeof(float));
        *b3 = h[7 * H + H * H];
    });
}

fedd_status fedd_trainer_grad(fedd_trainer *t, float wpsi, float wgrad, float *loss, float *gW1, float *gb1,
                              float *gW2, float *gb2, float *gw3, float *gb3) {
    if (!t || !loss) return FEDD_ERR_ARG;
    return tguard(t, [&] {
        FEDD_CUDA(cudaSetDevice(t->device));
        const int H = t->H;
        tr_workspace(t, t->n);
        std::vector<int64_t> id(t->n);
        for (int64_t i = 0; i < t->n; i++) id[i] = i;
        FEDD_CUDA(cudaMemcpy(t->idx.p, id.data(), t->n * sizeof(int64_t), cudaMemcpyHostToDevice));
        float b3 = 0;
        FEDD_CUDA(cudaMemcpy(&b3, t->par.p + 7 * H + H * H, sizeof b3, cudaMemcpyDeviceToHost));
        float L = tr_forward_backward(t, t->n, wpsi, wgrad, b3);
        *loss = L / (float)t->n;
        std::vector<float> g(t->nparams());
        FEDD_CUDA(cudaMemcpy(g.data(), t->grad.p, g.size() * sizeof(float), cudaMemcpyDeviceToHost));
        const float r = 1.0f / (float)t->n;
        for (auto &v : g) v *= r;
        if (gW1) std::memcpy(gW1, g.data(), 4 * H * sizeof(float));
        if (gb1) std::memcpy(gb1, g.data() + 4 * H, H * sizeof(float));
        if (gW2) std::memcpy(gW2, g.data() + 5 * H, (size_t)H * H * sizeof(float));
        if (gb2) std::memcpy(gb2, g.data() + 5 * H + H * H, H * sizeof(float));
        if (gw3) std::memcpy(gw3, g.data() + 6 * H + H * H, H * sizeof(float));
        if (gb3) *gb3 = g[7 * H + H * H];
    });
}

fedd_status fedd_trainer_run(fedd_trainer *t, int32_t steps, int64_t batch, float lr, float wpsi, float wgrad,
                             uint64_t seed, float *last_loss) {
    if (!t || steps < 0 || batch <= 0 || batch > t->n) return FEDD_ERR_ARG;
    return tguard(t, [&] {
        FEDD_CUDA(cudaSetDevice(t->device));
        const int H = t->H;
        tr_workspace(t, batch);
        if (t->perm.size() != (size_t)t->n || t->rng != seed) {
            t->perm.resize(t->n);
            for (int64_t i = 0; i < t->n; i++) t->perm[i] = i;
            t->rng = seed;
            t->cursor = t->n;
        }
        float L = 0;
        for (int it = 0; it < steps; it++) {
            if (t->cursor + batch > t->n) {  // reshuffle (Fisher-Yates, seeded)
                uint64_t st = t->rng ^ (0x5851F42D4C957F2DULL * (uint64_t)(t->step + 1));
                for (int64_t i = t->n - 1; i > 0; i--) {
                    int64_t j = (int64_t)(sm64(st) % (uint64_t)(i + 1));
                    std::swap(t->perm[i], t->perm[j]);
                }
                t->cursor = 0;
            }
            FEDD_CUDA(cudaMemcpy(t->idx.p, t->perm.data() + t->cursor, batch * sizeof(int64_t),
                                 cudaMemcpyHostToDevice));
            t->cursor += batch;
            float b3 = 0;
            FEDD_CUDA(cudaMemcpy(&b3, t->par.p + 7 * H + H * H, sizeof b3, cudaMemcpyDeviceToHost));
            L = tr_forward_backward(t, batch, wpsi, wgrad, b3) / (float)batch;
            t->step++;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.0f - std::pow(b1, (float)t->step), c2 = 1.0f - std::pow(b2, (float)t->step);
            const int np = t->nparams();
            k_adam<<<ceil_div(np, 256), 256>>>(t->par.p, t->grad.p, t->m1.p, t->m2.p, np, lr, b1, b2, 1e-8f, c1, c2,
                                               1.0f / (float)batch);
            FEDD_CUDA(cudaGetLastError());
        }
        FEDD_CUDA(cudaDeviceSynchronize());
        if (last_loss) *last_loss = L;
    });
}

fedd_status fedd_trainer_destroy(fedd_trainer *t) {
    if (!t) return FEDD_ERR_ARG;
    cudaSetDevice(t->device);
    delete t;
    return FEDD_OK;
}

}  // extern "C"
