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
#include "tcgen05.cuh"

namespace fedd {
namespace {

constexpr int kH = 64;        // tensor-core path width

// bf16 hi part of (x, y) and the bf16 rounding of the remainders: x ~ hi + lo
// to about 16 significant bits; x goes to the low half of each word (the
// lower K index of a K-major operand)
__device__ __forceinline__ void split_bf16(float x, float y, uint32_t &hi, uint32_t &lo) {
    uint32_t h, l;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(y), "f"(x));
    const float xh = __uint_as_float(h << 16), yh = __uint_as_float(h & 0xffff0000u);
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(l) : "f"(y - yh), "f"(x - xh));
    hi = h;
    lo = l;
}

// ---- quadrature-point derivatives on the fifth-generation tensor cores ------
// Tiles of 128 quadrature points (M = 128: point r of the tile in TMEM lane
// r), two threads per point: thread (r, h) of the 256 works on hidden units
// [32 h, 32 h + 32) (warps h * 4 .. h * 4 + 3 reach TMEM lanes 0-127).  With
// s1 = sigmoid(z1), t1 = s1 (1 - s1), D_k = W2 (s1 * W1[:, k]),
// s2 = sigmoid(z2), t2 = s2 (1 - s2):
//   dnet/dx_k       = sum_j w3_j s2_j D_kj
//   d2net/dx_k dx_l = sum_j w3_j t2_j D_kj D_lj + sum_i beta_i t1_i W1_ik W1_il,
//   beta = W2^T (w3 * s2)   (the backward product replaces the forward
//                            second-derivative channels).
// Layer 1 runs on the CUDA cores, its weights read from the constant bank.
// Its NC = 1 + NA channels (h1 = sp(z1), and s1 * W1[:, k] for the NA active
// inputs), split into bf16 hi + lo parts, are the A operands (K-major,
// 128 x 64) of layer 2: tcgen05.mma kind::f16 with W2 (bf16) as B and FP32
// accumulators in TMEM, 64 columns per channel.  The layer-2 epilogue reads
// them back, forms G and the first Hessian term, and writes w3 * s2 (hi +
// lo) as the A operand of the backward product beta = W2^T (w3 s2), which
// accumulates in channel 0's columns; the second Hessian term follows from
// beta and the t1 kept in registers.  The two threads of a point add their
// partial sums through shared memory.  One thread issues the MMAs and
// commits them to an mbarrier; every wait is bounded.
constexpr int kQT = 128;                      // points per tile
constexpr int kQThreads = 2 * kQT;            // threads per CTA: two per point
constexpr int kMA = kQT * kH * 2;             // bytes of one 128 x 64 bf16 operand (4 K steps of 4,096)
constexpr int kMB = kH * kH * 2;              // bytes of one 64 x 64 bf16 operand (4 K steps of 2,048)
constexpr uint32_t kMlpWaitPolls = 1u << 20;  // bounded MMA waits (each poll sleeps ~32 ns)

// byte offset of the 8-element chunk kc (K = 8 kc .. 8 kc + 7) of row r in a
// K-major unswizzled bf16 operand: 8-row x 16-byte core matrices, the two of
// one K step (16) 128 B apart (LBO), row groups 256 B apart (SBO), K steps
// `step` bytes apart
__host__ __device__ constexpr int mlp_off(int r, int kc, int step) {
    return (kc >> 1) * step + (r >> 3) * 256 + (kc & 1) * 128 + (r & 7) * 16;
}
// shared memory: the channels' A operands (hi, lo), W2 and W2^T as B, mbarrier + TMEM address
template <int NA> __host__ __device__ constexpr size_t mlp_smem() {
    return (size_t)(1 + NA) * 2 * kMA + 2 * (size_t)kMB + 16;
}
template <int NA> __host__ __device__ constexpr uint32_t mlp_tmem_cols() {
    return (1 + NA) * 64 <= 128 ? 128u : ((1 + NA) * 64 <= 256 ? 256u : 512u);
}

template <int NA>
__global__ void __launch_bounds__(kQThreads) k_mlp_qp_tc(MLPDev m, const float *__restrict__ inv, int64_t nqp,
                                                         QPDerivs *out, uint8_t *fb, int *fb_count, int *err) {
    constexpr int NC = 1 + NA, NH = NA * (NA + 1) / 2;
    constexpr uint32_t kCols = mlp_tmem_cols<NA>();
    static_assert(NC >= 2 || NA == 1, "channels");
    extern __shared__ __align__(1024) uint8_t ms[];
    uint8_t *sA = ms;                  // [channel][hi, lo][kMA]; after layer 2 channel 0 holds w3 s2
    uint8_t *sB1 = ms + NC * 2 * kMA;  // W2 as B: row j, K = i
    uint8_t *sB2 = sB1 + kMB;          // W2^T as B: row i, K = j
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sB2 + kMB);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
    // the upper threads' partial sums (channel 1's operand, free once layer 2 is done)
    float *sPart = reinterpret_cast<float *>(sA + 2 * kMA);
    const int tid = threadIdx.x, w = tid >> 5, r = tid & (kQT - 1), hh = tid >> 7;
    const MlpConst &c = m.c;
    const uint16_t *W2 = static_cast<const uint16_t *>(m.W2);
    for (int t = tid; t < kH * 8; t += kQThreads) {
        const int n = t >> 3, kc = t & 7;
        uint32_t b1w[4], b2w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k0 = 8 * kc + 2 * q;
            b1w[q] = (uint32_t)W2[n * kH + k0] | ((uint32_t)W2[n * kH + k0 + 1] << 16);
            b2w[q] = (uint32_t)W2[k0 * kH + n] | ((uint32_t)W2[(k0 + 1) * kH + n] << 16);
        }
        *reinterpret_cast<uint4 *>(sB1 + mlp_off(n, kc, 2048)) = make_uint4(b1w[0], b1w[1], b1w[2], b1w[3]);
        *reinterpret_cast<uint4 *>(sB2 + mlp_off(n, kc, 2048)) = make_uint4(b2w[0], b2w[1], b2w[2], b2w[3]);
    }
    if (w == 0) tc::tmem_alloc(tslot, kCols);
    if (tid == 0) tc::mbar_init(mbar, 1);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t trow = tmem + ((uint32_t)(32 * (w & 3)) << 16);  // this warp's 32 TMEM lanes
    constexpr uint32_t idesc = tc::idesc_bf16(kQT, kH);
    const uint32_t aBase = tc::smem_u32(sA), b1Base = tc::smem_u32(sB1), b2Base = tc::smem_u32(sB2);
    const int64_t ntiles = (nqp + kQT - 1) / kQT;
    uint32_t phase = 0;
    bool ok = true;
    // this thread's invariants, loaded one tile ahead
    auto load_inv = [&](int64_t tile) {
        const int64_t qq = tile * kQT + r;
        return qq < nqp ? reinterpret_cast<const float4 *>(inv)[qq] : make_float4(3.f, 1.f, 1.f, 1.f);
    };
    float4 v_next = load_inv(blockIdx.x);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t q = tile * kQT + r;
        bool inside = q < nqp;
        const float4 v4 = v_next;
        if (tile + gridDim.x < ntiles) v_next = load_inv(tile + gridDim.x);
        const float a4[4] = {v4.x, v4.y, v4.z, v4.w};
        // inputs, and the chain factors dx_k / dinv_k, d2x_k / dinv_k2 of the active ones
        float x[4], dk[NA], d2k[NA];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            inside = inside && a4[k] >= m.inv_lo[k] && a4[k] <= m.inv_hi[k];
            float d, h;
            x[k] = mlp_input(m, k, a4[k], d, h);
#pragma unroll
            for (int a = 0; a < NA; a++)
                if (c.act[a] == k) {
                    dk[a] = d;
                    d2k[a] = h;
                }
        }
        // layer 1 over this thread's 32 units, eight at a time: one 16-byte
        // chunk per channel and part
        float t1[kH / 2];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            float v[NC][8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = 32 * hh + 8 * g + u;
                float z = c.b1[i];
#pragma unroll
                for (int k = 0; k < 4; k++) z = fmaf(c.W1[i][k], x[k], z);
                // softplus and sigmoid from one exponential, e = exp(-|z|) in
                // (0, 1]: sp = max(z, 0) + log(1 + e), s = 1 / (1 + e) or e / (1 + e);
                // fast-math log and reciprocal (a few ulp, below the bf16 hi + lo
                // rounding of the layer-2 operand)
                const float e1 = __expf(-fabsf(z)), r1 = __fdividef(1.0f, 1.0f + e1);
                const float s1 = z >= 0.0f ? r1 : e1 * r1;
                t1[8 * g + u] = s1 * (1.0f - s1);
                v[0][u] = fmaxf(z, 0.0f) + __logf(1.0f + e1);
#pragma unroll
                for (int a = 0; a < NA; a++) v[1 + a][u] = s1 * c.Wact[a][i];
            }
            const int o = mlp_off(r, 4 * hh + g, 4096);
#pragma unroll
            for (int ch = 0; ch < NC; ch++) {
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int p = 0; p < 4; p++) split_bf16(v[ch][2 * p], v[ch][2 * p + 1], hw[p], lw[p]);
                *reinterpret_cast<uint4 *>(sA + (2 * ch) * kMA + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(sA + (2 * ch + 1) * kMA + o) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int ch = 0; ch < NC; ch++)
#pragma unroll
                for (int part = 0; part < 2; part++)
#pragma unroll
                    for (int ks = 0; ks < 4; ks++)
                        tc::mma_bf16(tmem + 64 * ch, tc::smem_desc(aBase + (2 * ch + part) * kMA + ks * 4096, 128, 256),
                                     tc::smem_desc(b1Base + ks * 2048, 128, 256), idesc, (part | ks) != 0);
            tc::commit(mbar);
        }
        const bool done = tc::mbar_wait(mbar, phase, kMlpWaitPolls);
        phase ^= 1u;
        if (__syncthreads_or(!done)) {
            ok = false;
            break;
        }
        tc::fence_after_sync();
        // layer-2 epilogue over this thread's 32 units, 16 at a time; w3 s2
        // (hi + lo) becomes channel 0's operand (layer 2 has completed)
        float G[NA], Hh[NH];
#pragma unroll
        for (int a = 0; a < NA; a++) G[a] = 0.0f;
#pragma unroll
        for (int a = 0; a < NH; a++) Hh[a] = 0.0f;
#pragma unroll
        for (int jj = 0; jj < 2; jj++) {
            const int jc = 2 * hh + jj;
            float z2[16], dd[NA][16], vv[16];
            tc::tmem_ld16(trow + 16 * jc, z2);
#pragma unroll
            for (int a = 0; a < NA; a++) tc::tmem_ld16(trow + 64 * (1 + a) + 16 * jc, dd[a]);
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const int j = 16 * jc + u;
                // sigmoid with a fast reciprocal (a few ulp, below the bf16
                // hi + lo rounding of the backward product's operand)
                const float zz = z2[u] + c.b2[j];
                const float e2 = __expf(-fabsf(zz)), r2 = __fdividef(1.0f, 1.0f + e2);
                const float s2 = zz >= 0.0f ? r2 : e2 * r2;
                const float cs = c.w3[j] * s2, ct = c.w3[j] * (s2 * (1.0f - s2));
                int ab = 0;
#pragma unroll
                for (int a = 0; a < NA; a++) {
                    G[a] = fmaf(cs, dd[a][u], G[a]);
                    const float cd = ct * dd[a][u];
#pragma unroll
                    for (int b = a; b < NA; b++, ab++) Hh[ab] = fmaf(cd, dd[b][u], Hh[ab]);
                }
                vv[u] = cs;
            }
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int p = 0; p < 4; p++) split_bf16(vv[8 * hf + 2 * p], vv[8 * hf + 2 * p + 1], hw[p], lw[p]);
                const int o = mlp_off(r, 2 * jc + hf, 4096);
                *reinterpret_cast<uint4 *>(sA + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(sA + kMA + o) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int part = 0; part < 2; part++)
#pragma unroll
                for (int ks = 0; ks < 4; ks++)
                    tc::mma_bf16(tmem, tc::smem_desc(aBase + part * kMA + ks * 4096, 128, 256),
                                 tc::smem_desc(b2Base + ks * 2048, 128, 256), idesc, (part | ks) != 0);
            tc::commit(mbar);
        }
        const bool done2 = tc::mbar_wait(mbar, phase, kMlpWaitPolls);
        phase ^= 1u;
        if (__syncthreads_or(!done2)) {
            ok = false;
            break;
        }
        tc::fence_after_sync();
        // sum_i beta_i t1_i W1_ik W1_il over this thread's units
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
            const int ic = 2 * hh + ii;
            float bt[16];
            tc::tmem_ld16(trow + 16 * ic, bt);
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const int i = 16 * ic + u;
                const float b = bt[u] * t1[16 * ii + u];
                int ab = 0;
#pragma unroll
                for (int a = 0; a < NA; a++) {
                    const float bw = b * c.Wact[a][i];
#pragma unroll
                    for (int b2 = a; b2 < NA; b2++, ab++) Hh[ab] = fmaf(bw, c.Wact[b2][i], Hh[ab]);
                }
            }
        }
        // the upper thread of each point hands its partial sums to the lower one
        if (hh == 1) {
#pragma unroll
            for (int a = 0; a < NA; a++) sPart[(NA + NH) * r + a] = G[a];
#pragma unroll
            for (int a = 0; a < NH; a++) sPart[(NA + NH) * r + NA + a] = Hh[a];
        }
        __syncthreads();
        if (hh == 0) {
#pragma unroll
            for (int a = 0; a < NA; a++) G[a] += sPart[(NA + NH) * r + a];
#pragma unroll
            for (int a = 0; a < NH; a++) Hh[a] += sPart[(NA + NH) * r + NA + a];
        }
        if (hh == 0 && q < nqp) {
            // scatter to the packed (I1, J, I4a, I4b) layout with static indices
            QPDerivs d;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float v = 0.0f;
#pragma unroll
                for (int a = 0; a < NA; a++)
                    if (c.act[a] == k) v = m.out_scale * G[a] * dk[a];
                d.d1[k] = v;
            }
            int kl = 0;
#pragma unroll
            for (int k = 0; k < 4; k++)
#pragma unroll
                for (int l = k; l < 4; l++, kl++) {
                    // packed symmetric index of (k, l), k <= l: 00,01,02,03,11,12,13,22,23,33
                    float v = 0.0f;
                    int ab = 0;
#pragma unroll
                    for (int a = 0; a < NA; a++)
#pragma unroll
                        for (int b = a; b < NA; b++, ab++)
                            if (c.act[a] == k && c.act[b] == l)
                                v = m.out_scale * (Hh[ab] * dk[a] * dk[b] + (a == b ? G[a] * d2k[a] : 0.0f));
                    d.d2[kl] = v;
                }
            out[q] = d;
            fb[q] = inside ? 0 : 1;
            if (!inside) atomicAdd(fb_count, 1);
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (!ok) {
        // the MMAs did not complete in time: report it, give them a second
        // bounded wait, then free the tensor memory all the same
        if (tid == 0) set_dev_error(err, kDevTimeout);
        tc::mbar_wait(mbar, phase ^ 1u, kMlpWaitPolls);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (w == 0) tc::tmem_dealloc(tmem, kCols);
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


template <int NA>
void launch_mlp_qp_tc(const MLPDev &m, const float *inv, int64_t nqp, QPDerivs *out, uint8_t *fallback, int *d_count,
                      int *d_err, cudaStream_t s) {
    constexpr size_t smem = mlp_smem<NA>();
    // CTAs per SM: shared memory (and, for two active inputs, the 512 TMEM columns) allow two up to NA = 2
    const int per_sm = NA <= 2 ? 2 : 1;
    const unsigned grid = (unsigned)std::min<int64_t>(ceil_div(nqp, kQT), (int64_t)sms() * per_sm);
    FEDD_CUDA(cudaFuncSetAttribute(k_mlp_qp_tc<NA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_mlp_qp_tc<NA><<<grid, kQThreads, smem, s>>>(m, inv, nqp, out, fallback, d_count, d_err);
}

}  // namespace

void launch_mlp_qp(const MLPDev &m, const LawParams &law, const float *inv, int64_t nqp, QPDerivs *out,
                   uint8_t *fallback, int *d_count, int *d_err, cudaStream_t s, LaunchCounter &lc) {
    (void)law;
    if (nqp == 0) return;
    if (m.hidden == kH && m.c.nact > 0) {
        switch (m.c.nact) {
        case 1: launch_mlp_qp_tc<1>(m, inv, nqp, out, fallback, d_count, d_err, s); break;
        case 2: launch_mlp_qp_tc<2>(m, inv, nqp, out, fallback, d_count, d_err, s); break;
        case 3: launch_mlp_qp_tc<3>(m, inv, nqp, out, fallback, d_count, d_err, s); break;
        default: launch_mlp_qp_tc<4>(m, inv, nqp, out, fallback, d_count, d_err, s); break;
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
