// k_ns.cu -- P2-P1 Taylor-Hood Navier-Stokes Jacobian + residual.
//
// Element math of AssembleFENavierStokes
// (feddlib/core/AceFemAssembly/specific/AssembleFENavierStokes_def.hpp):
//   A  (Laplacian, :149-196), N (advection, :227-298),
//   W  (Newton term, :301-369), B / B^T (divergence, :373-461),
//   J = nu rho A - B - B^T + rho N (+ rho W for Newton)      :66-112
//   r = (nu rho A - B - B^T + rho N) x  (coeff = 1)          :199-224
// For affine elements each term is a contraction of a few per-element
// coefficients with reference integrals (tables.cpp):
//   A_ab  = sum_s Gs_s KS[a][b][s],           Gs = |det B| B^-1 B^-T
//   N_ab  = sum_{c,k} uT[c][k] T[c][a][b][k], uT = |det B| B^-1 u_k
//   W_(ai)(bj) = sum_m g[j][m][i] R[a][b][m],  g = |det B| grad u at vertex m
//   Bd_p(bd) = sum_c Bs[d][c] Y[b][p][c],     Bs = |det B| B^-1
// A record kernel (one thread per element, FP64 geometry) writes these
// coefficients; the row kernels (one warp per node) contract them for the
// node's row and accumulate in shared memory, then write each CSR value once.
#include "kernels.cuh"
#include "tcgen05.cuh"

namespace fedd {
namespace {

// record layout (floats, 16-byte aligned groups)
// [0, kRecVel) holds everything the velocity rows read besides NA, so one
// 336-byte bulk copy stages it
constexpr int kRecG = 0;     // g[j][12] = (m*3 + i)
constexpr int kRecBS = 36;   // Bs[d][4] (c < 3)
constexpr int kRecU = 48;    // u[30] node-wise
constexpr int kRecP = 78;    // p[4]
constexpr int kRecVel = 84;
constexpr int kRecUT = 84;   // uT[c][12] = |det B| (B^-1 u_k)_c   (k < 10)
constexpr int kRecGS = 120;  // Gs[6]
constexpr int kRecNA = 128;  // NA[a][b] = nu rho A_ab + rho N_ab (100 floats)
static_assert(kNSRecord == kRecNA + 100, "record size");

// device table layout (floats)
// T is stored per row node a and chunk of four k as [a][kc][lane][4] with
// lane = 3 b + c (30 of 32 used), so that the warp's 16-byte reads of one
// chunk cover 512 contiguous bytes (no bank conflicts).
constexpr int kTabT = 0;        // T[a][kc][lane][4]  3840
constexpr int kTabKS = 3840;    // KS[a][b][6]        600
constexpr int kTabR = 4440;     // R[a][b][4]         400
constexpr int kTabY = 4840;     // Y[b][p][4] (c < 3) 160
constexpr int kTabSize = 5000;
constexpr int kVelTab = 560;    // floats of tables the velocity-row kernel keeps in shared memory (R, Y)

__constant__ float c_dv[4][10][3];



// ---- the record stage: coefficients, and NA on the fifth-generation tensor cores
// NA_e[n] = sum_kk X_e[kk] Y[kk][n], n = 10 a + b, with
//   X_e = (uT[c][k] at kk = 10 c + k for c < 3, k < 10; Gs[s] at kk = 30 + s)
//   Y   = (rho T[c][a][b][k]; nu rho KS[a][b][s])
// is a GEMM of (elements x 36) by (36 x 100), K padded to 40 and N to 112.
// One kernel computes each element's record (one thread per element, FP64
// geometry) and, for every tile of 128 elements (M = 128, element i of the
// tile in TMEM lane i), that tile's NA: the threads split X into TF32 hi +
// lo parts and write them to shared memory as K-major operands, one thread
// issues tcgen05.mma kind::tf32 for hi hi + hi lo + lo hi (5 K steps of 8,
// FP32 accumulation in TMEM: about FP32 accuracy) and commits to an
// mbarrier, and each warp reads its 32 rows of NA back from TMEM.  A CTA
// (one per SM, persistent) runs four independent groups of 128 threads,
// each with its own tiles, A region, mbarrier, named barrier and 128 TMEM
// columns; the groups share one copy of Y's hi and lo parts, built once.
constexpr int kNAK = 40;                     // K: 36 coefficients padded to 5 steps of 8
constexpr int kNAN = 112;                    // N: 100 (a, b) pairs padded to a multiple of 16
constexpr int kRecTile = 128;                // M: elements per tile = threads per group
constexpr int kRecGroups = 4;                // groups per CTA
constexpr int kRecThreads = kRecGroups * kRecTile;
constexpr int kNAStepA = kRecTile * 32;      // bytes of one K step (8 TF32) of the A operand
constexpr int kNAStepB = kNAN * 32;          // ... of the B operand
constexpr int kNABytesA = 5 * kNAStepA;      // 20,480 per part
constexpr int kNABytesB = 5 * kNAStepB;      // 17,920 per part
constexpr int kRecWarpBytes = 2 * kNABytesA / 4;  // each warp's share of its group's A region between the MMAs
// Shared memory: B (hi, lo), then each group's A region (hi, lo), which
// between the MMAs holds its warps' record and NA staging, then the groups'
// mbarriers and the TMEM address: 199,728 bytes, one CTA (16 warps) per SM.
constexpr int kRecAOff = 2 * kNABytesB;
constexpr int kRecBarOff = kRecAOff + kRecGroups * 2 * kNABytesA;
constexpr size_t kRecSmem = (size_t)kRecBarOff + 8 * kRecGroups + 16;
constexpr uint32_t kNAWaitPolls = 1u << 20;  // bounded wait for the MMAs (each poll sleeps ~32 ns)
static_assert(kRecGS == kRecUT + 36 && kRecNA == kRecGS + 8, "uT, Gs and NA are laid out back to back");
static_assert(kRecWarpBytes >= 32 * 17 * 16 && kRecWarpBytes >= 32 * 68 * 4, "per-warp staging fits");
static_assert(kRecSmem <= 227 * 1024 && kRecGroups * 128 <= 512, "one CTA per SM: shared memory and TMEM");

// byte offset of (row, k) in a K-major, unswizzled operand: 8-row x 16-byte
// core matrices, the two of one K step 128 B apart (LBO), row groups 256 B
// apart (SBO), K steps `step` bytes apart
__device__ __forceinline__ int na_off(int row, int k, int step) {
    return (k >> 3) * step + (row >> 3) * 256 + ((k >> 2) & 1) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

// barrier over the 128 threads of group g (named barrier 1 + g)
__device__ __forceinline__ void group_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }
// ... which also returns whether any of them passed v != 0
__device__ __forceinline__ bool group_sync_or(int g, bool v) {
    uint32_t r;
    asm volatile("{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, %2, 128, p;\nselp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r)
                 : "r"((uint32_t)v), "r"(1 + g)
                 : "memory");
    return r != 0;
}

// elements [e_begin, e_end)
__global__ void __launch_bounds__(kRecThreads, 1) k_ns_record(const double *__restrict__ xyz, const int32_t *__restrict__ conn2,
                                                             const int32_t *__restrict__ conn1, int64_t ne,
                                                             const double *__restrict__ u, const double *__restrict__ p,
                                                             float *rec, int *err, int64_t e_begin, int64_t e_end,
                                                             const float *__restrict__ gtab, float visc_dens, float dens) {
    extern __shared__ __align__(1024) uint8_t rs[];
    const int tid = threadIdx.x, gi = tid >> 7, gt = tid & (kRecTile - 1), wl = (tid >> 5) & 3, lane = tid & 31;
    uint8_t *sBh = rs, *sBl = rs + kNABytesB;
    uint8_t *sAh = rs + kRecAOff + gi * 2 * kNABytesA, *sAl = sAh + kNABytesA;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(rs + kRecBarOff) + gi;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(rs + kRecBarOff + 8 * kRecGroups);
    uint8_t *sW = sAh + wl * kRecWarpBytes;  // this warp's staging, between the MMAs
    // B = Y^T: row n, column kk
    for (int t = tid; t < kNAN * kNAK; t += kRecThreads) {
        const int n = t / kNAK, kk = t - kNAK * (t / kNAK);
        float y = 0.0f;
        if (n < 100) {
            const int a = n / 10, b = n % 10;
            if (kk < 30) {
                const int c = kk / 10, k = kk % 10;
                // T[a][kc][lane = 3 b + c][k % 4] in the device table
                y = dens * gtab[kTabT + ((a * 3 + k / 4) * 32 + 3 * b + c) * 4 + k % 4];
            } else if (kk < 36) {
                y = visc_dens * gtab[kTabKS + (a * 10 + b) * 6 + (kk - 30)];
            }
        }
        const uint32_t h = to_tf32(y);
        const int o = na_off(n, kk, kNAStepB);
        *reinterpret_cast<uint32_t *>(sBh + o) = h;
        *reinterpret_cast<uint32_t *>(sBl + o) = to_tf32(y - __uint_as_float(h));
    }
    if (tid < 32) tc::tmem_alloc(tslot, 128 * kRecGroups);
    if (gt == 0) tc::mbar_init(mbar, 1);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot + 128u * gi;                  // this group's 128 columns
    const uint32_t trow = tmem + ((uint32_t)(32 * wl) << 16);  // this warp's 32 TMEM lanes
    constexpr uint32_t idesc = tc::idesc_tf32(kRecTile, kNAN);
    const int64_t ntiles = (e_end - e_begin + kRecTile - 1) / kRecTile;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t tile = (int64_t)blockIdx.x * kRecGroups + gi; tile < ntiles; tile += (int64_t)gridDim.x * kRecGroups) {
        // every thread stays for the collective steps; threads past the range
        // recompute the last element and store nothing
        const int64_t e_lane = e_begin + tile * kRecTile + gt;
        const int64_t e = e_lane < e_end ? e_lane : e_end - 1;
        float Bi[9];
        const float det = d2f_rn(geometry_fp64(xyz, conn2[e], conn2[ne + e], conn2[2 * ne + e], conn2[3 * ne + e], Bi));
        if (!(det > 0.0f) && !(det < 0.0f)) set_dev_error(err, kDevBadDet);
        const float ad = fabsf(det);
        float ue[30];
#pragma unroll
        for (int k = 0; k < 10; k++) {
            const int32_t node = conn2[(int64_t)k * ne + e];
            const double *up = u + 3 * (int64_t)node;
            ue[3 * k] = d2f_rn(up[0]);
            ue[3 * k + 1] = d2f_rn(up[1]);
            ue[3 * k + 2] = d2f_rn(up[2]);
        }
        float R[kRecNA];
#pragma unroll
        for (int k = 0; k < kRecNA; k++) R[k] = 0.0f;
        // uT[c][k] = |det| sum_d Binv[c][d] u_{k,d}
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int k = 0; k < 10; k++)
                R[kRecUT + 12 * c + k] = ad * (Bi[3 * c] * ue[3 * k] + Bi[3 * c + 1] * ue[3 * k + 1] + Bi[3 * c + 2] * ue[3 * k + 2]);
        // g[j][m][i] = |det| sum_c Binv[c][j] sum_k u_{k,i} dphi_ref_c(phi_k)(v_m)
#pragma unroll
        for (int m = 0; m < 4; m++) {
            float Hm[3][3];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float h = 0.0f;
#pragma unroll
                    for (int k = 0; k < 10; k++) h = fmaf(ue[3 * k + i], c_dv[m][k][c], h);
                    Hm[i][c] = h;
                }
#pragma unroll
            for (int j = 0; j < 3; j++)
#pragma unroll
                for (int i = 0; i < 3; i++)
                    R[kRecG + 12 * j + 3 * m + i] = ad * (Bi[j] * Hm[i][0] + Bi[3 + j] * Hm[i][1] + Bi[6 + j] * Hm[i][2]);
        }
        // Gs = |det| B^-1 B^-T (00,11,22,01,02,12)
        const int SC[6] = {0, 1, 2, 0, 0, 1}, SD[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int s = 0; s < 6; s++)
            R[kRecGS + s] = ad * (Bi[3 * SC[s]] * Bi[3 * SD[s]] + Bi[3 * SC[s] + 1] * Bi[3 * SD[s] + 1] +
                                  Bi[3 * SC[s] + 2] * Bi[3 * SD[s] + 2]);
#pragma unroll
        for (int d = 0; d < 3; d++)
#pragma unroll
            for (int c = 0; c < 3; c++) R[kRecBS + 4 * d + c] = ad * Bi[3 * c + d];
#pragma unroll
        for (int k = 0; k < 30; k++) R[kRecU + k] = ue[k];
#pragma unroll
        for (int k = 0; k < 4; k++) R[kRecP + k] = p ? d2f_rn(p[conn1[(int64_t)k * ne + e]]) : 0.0f;
        // the warp's 32 records (floats [0, kRecNA)) go out through shared
        // memory in two halves of 64 floats, so that each store instruction
        // writes two records' halves as contiguous 256-byte runs; rows of 17
        // chunks keep the 16-byte shared stores conflict-free
        float4 *sRec = reinterpret_cast<float4 *>(sW);
        const int64_t ew0 = e_lane - lane;
#pragma unroll
        for (int h = 0; h < 2; h++) {
#pragma unroll
            for (int k = 0; k < 16; k++)
                sRec[lane * 17 + k] = make_float4(R[64 * h + 4 * k], R[64 * h + 4 * k + 1], R[64 * h + 4 * k + 2],
                                                  R[64 * h + 4 * k + 3]);
            __syncwarp();
#pragma unroll 4
            for (int r = 0; r < 32; r += 2) {
                const int rr = r + (lane >> 4);
                const int64_t er = ew0 + rr;
                if (er < e_end) reinterpret_cast<float4 *>(rec + er * kNSRecord)[16 * h + (lane & 15)] = sRec[rr * 17 + (lane & 15)];
            }
            __syncwarp();
        }
        group_sync(gi);  // every warp's staging is done before the A operand overwrites it
#pragma unroll
        for (int q = 0; q < kNAK / 4; q++) {
            uint32_t hv[4], lv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int kk = 4 * q + i;
                const float v = kk < 30 ? R[kRecUT + 12 * (kk / 10) + kk % 10] : (kk < 36 ? R[kRecGS + kk - 30] : 0.0f);
                hv[i] = to_tf32(v);
                lv[i] = to_tf32(v - __uint_as_float(hv[i]));
            }
            const int o = na_off(gt, 4 * q, kNAStepA);
            *reinterpret_cast<uint4 *>(sAh + o) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
            *reinterpret_cast<uint4 *>(sAl + o) = make_uint4(lv[0], lv[1], lv[2], lv[3]);
        }
        tc::fence_proxy_async();
        group_sync(gi);
        if (gt == 0) {
            tc::fence_after_sync();
            const uint32_t aH = tc::smem_u32(sAh), aL = tc::smem_u32(sAl), bH = tc::smem_u32(sBh), bL = tc::smem_u32(sBl);
#pragma unroll
            for (int ks = 0; ks < 5; ks++) {
                const uint64_t ah = tc::smem_desc(aH + ks * kNAStepA, 128, 256), al = tc::smem_desc(aL + ks * kNAStepA, 128, 256);
                const uint64_t bh = tc::smem_desc(bH + ks * kNAStepB, 128, 256), bl = tc::smem_desc(bL + ks * kNAStepB, 128, 256);
                tc::mma_tf32(tmem, ah, bh, idesc, ks > 0);
                tc::mma_tf32(tmem, ah, bl, idesc, 1);
                tc::mma_tf32(tmem, al, bh, idesc, 1);
            }
            tc::commit(mbar);
        }
        const bool done = tc::mbar_wait(mbar, phase, kNAWaitPolls);
        phase ^= 1u;
        if (group_sync_or(gi, !done)) {
            ok = false;
            break;
        }
        tc::fence_after_sync();
        // NA rows out through the warp's staging: columns 0-63 (rows of 68
        // floats), then 64-99 (rows of 36); each store instruction writes
        // whole 256-byte (two rows) or 144-byte (three rows) runs of records
        float *sN = reinterpret_cast<float *>(sW);
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
            float v[16];
            tc::tmem_ld16(trow + 16 * ch, v);
#pragma unroll
            for (int i = 0; i < 16; i += 4)
                *reinterpret_cast<float4 *>(sN + lane * 68 + 16 * ch + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
        __syncwarp();
#pragma unroll 4
        for (int r = 0; r < 32; r += 2) {
            const int rr = r + (lane >> 4);
            const int64_t er = ew0 + rr;
            if (er < e_end)
                reinterpret_cast<float4 *>(rec + er * kNSRecord + kRecNA)[lane & 15] =
                    *reinterpret_cast<const float4 *>(sN + rr * 68 + 4 * (lane & 15));
        }
        __syncwarp();
#pragma unroll
        for (int ch = 4; ch < 7; ch++) {
            float v[16];
            tc::tmem_ld16(trow + 16 * ch, v);
#pragma unroll
            for (int i = 0; i < 16; i += 4)
                if (16 * ch + i < 100)
                    *reinterpret_cast<float4 *>(sN + lane * 36 + 16 * (ch - 4) + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
        __syncwarp();
        for (int r = 0; r < 32; r += 3) {
            const int rr = r + lane / 9, c4 = lane % 9;
            const int64_t er = ew0 + rr;
            if (lane < 27 && rr < 32 && er < e_end)
                reinterpret_cast<float4 *>(rec + er * kNSRecord + kRecNA + 64)[c4] =
                    *reinterpret_cast<const float4 *>(sN + rr * 36 + 4 * c4);
        }
        tc::fence_before_sync();
        group_sync(gi);
    }
    if (!ok) {
        // the MMAs did not complete in time: report it, give them a second
        // bounded wait, then free the tensor memory all the same
        if (gt == 0) set_dev_error(err, kDevTimeout);
        tc::mbar_wait(mbar, phase ^ 1u, kNAWaitPolls);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid < 32) tc::tmem_dealloc(*tslot, 128 * kRecGroups);
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// Lane (b, j) of one incidence with row node a: returns its share of
// (nu rho A_ab + rho N_ab) (the three lanes of b hold the c = j parts) and
// fills w[i] = W_(ai)(bj).
__device__ __forceinline__ float ns_lane_terms(const float *rec, const float *tab, int a, int b, int j,
                                               float visc_dens, float dens, float w[3]) {
    const float *T = tab + kTabT + (a * 96 + 3 * b + j) * 4;
    const float *U = rec + kRecUT + 12 * j;
    const float4 t0 = lds4(T), t1 = lds4(T + 128), t2 = lds4(T + 256);
    const float4 u0 = lds4(U), u1 = lds4(U + 4), u2 = lds4(U + 8);
    const float n = (u0.x * t0.x + u0.y * t0.y + u0.z * t0.z + u0.w * t0.w) +
                    (u1.x * t1.x + u1.y * t1.y + u1.z * t1.z + u1.w * t1.w) + (u2.x * t2.x + u2.y * t2.y);
    const float2 ks = *reinterpret_cast<const float2 *>(tab + kTabKS + (a * 10 + b) * 6 + 2 * j);
    const float2 gs = *reinterpret_cast<const float2 *>(rec + kRecGS + 2 * j);
    const float av = gs.x * ks.x + gs.y * ks.y;
    const float4 r = lds4(tab + kTabR + (a * 10 + b) * 4);
    const float *G = rec + kRecG + 12 * j;
    const float4 g0 = lds4(G), g1 = lds4(G + 4), g2 = lds4(G + 8);
    // g[j][m*3+i]: m0 = (g0.x,g0.y,g0.z) m1 = (g0.w,g1.x,g1.y) m2 = (g1.z,g1.w,g2.x) m3 = (g2.y,g2.z,g2.w)
    w[0] = g0.x * r.x + g0.w * r.y + g1.z * r.z + g2.y * r.w;
    w[1] = g0.y * r.x + g1.x * r.y + g1.w * r.z + g2.z * r.w;
    w[2] = g0.z * r.x + g1.y * r.y + g2.x * r.z + g2.w * r.w;
    return visc_dens * av + dens * n;
}

// -Bd_p(a,i) for B^T lane (i, p): the (0,1) entry of velocity row (a, i)
__device__ __forceinline__ float ns_bt(const float *rec, const float *tab, int a, int i, int p) {
    const float4 bs = lds4(rec + kRecBS + 4 * i);
    const float4 y = lds4(tab + kTabY + (a * 4 + p) * 4);
    return -(bs.x * y.x + bs.y * y.y + bs.z * y.z);
}

__device__ __forceinline__ float sum3_lanes(float part, int lane) {
    const int b = lane / 3, j = lane - 3 * b;
    int s1 = 3 * b + (j + 1) % 3, s2 = 3 * b + (j + 2) % 3;
    if (lane >= 30) { s1 = lane; s2 = lane; }
    float x1 = __shfl_sync(0xffffffffu, part, s1);
    float x2 = __shfl_sync(0xffffffffu, part, s2);
    return part + x1 + x2;
}

// Per velocity-row node, one 16-byte word: the first incidence (int64, x | y),
// the P1 node at the vertex (z, -1 for edge nodes or without a verified
// vertex map) and w = K | Kp << 8 | m << 16 (velocity and pressure
// neighbours, at most kMaxAdjacency = 255 each; incidences, at most 64).
__device__ __forceinline__ int64_t node_i0(int4 v) {
    return (int64_t)(((uint64_t)(uint32_t)v.y << 32) | (uint32_t)v.x);
}
__device__ __forceinline__ int node_k(int4 v) { return v.w & 255; }
__device__ __forceinline__ int node_kp(int4 v) { return (v.w >> 8) & 255; }
__device__ __forceinline__ int node_m(int4 v) { return (v.w >> 16) & 255; }

__global__ void k_ns_node_info(const int64_t *__restrict__ inc_ptr, const int64_t *__restrict__ adj_ptr,
                               const int64_t *__restrict__ padj_ptr, const int32_t *__restrict__ vmap, int64_t nn,
                               int4 *info) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int64_t i0 = inc_ptr[n];
    const int m = (int)(inc_ptr[n + 1] - i0);
    const int K = (int)(adj_ptr[n + 1] - adj_ptr[n]), Kp = (int)(padj_ptr[n + 1] - padj_ptr[n]);
    info[n] = make_int4((int)(uint32_t)(uint64_t)i0, (int)(uint32_t)((uint64_t)i0 >> 32), vmap ? vmap[n] : -1,
                        K | (Kp << 8) | (m << 16));
}

// velocity rows: block (0,0) and (0,1) values and the velocity residual.
// One warp per row node a.  Each incidence's record head (g, Bs, u, p), the
// 48-byte window holding NA[a][:] and its slot map are staged into a ring of
// kVRing shared-memory slots, kVRing - 1 incidences ahead, by one 16-byte
// cp.async per lane (lanes 0-20 the head, 21-23 the NA window, 24 the slot
// map): 400 bytes instead of the whole 912-byte record.
// Shared-memory accumulators form three planes, one per row component i,
// each holding (column slot, j) at 3 slot + j and the pressure columns after
// the 3 K velocity ones; a lane's update of an incidence is three 4-byte
// read-modify-writes (32-bit shared accesses run at twice the bytes per clock
// of 16-byte ones on this part, and no padding word is moved).
// The incidence loop is unrolled by the ring size so every ring offset is an
// immediate; idle lanes write a scratch word instead of branching.
// With a generalized-Newtonian viscous stage (the dense element matrix with
// rows padded to 32 floats, kGNStride floats per element) each slot also
// holds the element's three rows 3 a + i (lanes 0-23, second copy) and an
// 8-float window holding its residual entries 3 a .. 3 a + 2 (lanes 24-25),
// which the lanes fold into the same accumulation: no separate pass re-reads
// and re-writes the rows.
constexpr int kVRing = 4;
constexpr int kVStage = 100;  // floats per ring slot: record head 84 | NA window 12 | slot map 16 B
constexpr int kVNA = kRecVel, kVSlots = kRecVel + 12;
constexpr int kVGn = kVStage, kVGnRes = kVStage + 96, kVStageGn = kVStage + 104;
static_assert(kVSlots + 4 == kVStage && kRecVel % 4 == 0, "ring slot layout: lane L copies floats [4 L, 4 L + 4)");

// stage incidence t (of m) into ring slot `slot` (a constant after unrolling);
// every call commits one group, empty past the node's last incidence, so the
// wait counts hold.  src_lane = 4 lane floats into the record for head lanes,
// kRecNA + 4 (lane - 21) for NA-window lanes; dst_lane = ring + 4 lane.
template <bool GN>
__device__ __forceinline__ void stage_vel(float *dst_lane, int slot, int t, int m, const IncList &il,
                                          const float *__restrict__ rec, int src_lane, int kind,
                                          const uint8_t *__restrict__ slots_node, const float *__restrict__ gstage,
                                          int lane) {
    constexpr int kStg = GN ? kVStageGn : kVStage;
    if (t < m) {
        // one shuffle when the node's list fits the low word (warp-uniform)
        const uint32_t ea = m <= 32 ? __shfl_sync(0xffffffffu, il.lo, t & 31) : incidence_at(il, t);
        const int a = (int)(ea & 15u);
        // NA[a][0..9] starts 8 bytes into a 16-byte boundary when a is odd
        const float *r = rec + (size_t)(ea >> 4) * kNSRecord + src_lane + (kind == 1 ? 10 * a - 2 * (a & 1) : 0);
        const void *src = kind == 2 ? static_cast<const void *>(slots_node + t * kSlotStride) : static_cast<const void *>(r);
        if (kind < 3) cp_async16(dst_lane + slot * kStg, src);
        if (GN && lane < 26) {
            const float *Ke = gstage + (size_t)(ea >> 4) * kGNStride;
            // lane < 24: row 3 a + (lane >> 3), chunk lane & 7; lanes 24, 25: the residual window
            const float *g = lane < 24 ? Ke + 32 * (3 * a + (lane >> 3)) + 4 * (lane & 7)
                                       : Ke + kGNRes + 4 * ((3 * a) >> 2) + 4 * (lane - 24);
            cp_async16(dst_lane - 4 * lane + slot * kStg + (lane < 24 ? kVGn + 4 * lane : kVGnRes + 4 * (lane - 24)), g);
        }
    }
    cp_async_commit();
}

template <bool GN>
__global__ void __launch_bounds__(512, 2) k_ns_vel_rows(const int4 *__restrict__ ninfo, const uint32_t *__restrict__ inc,
                                                        const uint8_t *__restrict__ slots, const float *__restrict__ rec,
                                                        const float *__restrict__ gtab, const int64_t *__restrict__ rowptr00,
                                                        const int64_t *__restrict__ rowptr01, double *vals00, double *vals01,
                                                        double *res_u, int64_t nnodes, float dens, int newton, int max_adj,
                                                        int max_padj, int64_t n_begin, int fused,
                                                        const int64_t *__restrict__ rowptr10, double *vals10, double *res_p,
                                                        const float *__restrict__ gstage, unsigned long long *work,
                                                        NSCoeff co) {
    constexpr int kStg = GN ? kVStageGn : kVStage;
    extern __shared__ __align__(16) float smem[];
    // the W table scaled by the Newton weight (rho, or 0 for the Picard form)
    // and the B^T table negated: sR = wn R[a][b][4], sY = -Y[a][p][4]; the
    // diagonal part NA comes with each record
    float *sR = smem, *sY = smem + 400;
    static_assert(kTabY == kTabR + 400 && kVelTab == 560, "R and Y are adjacent");
    const float wn = newton ? dens : 0.0f;
    for (int t = threadIdx.x; t < kVelTab; t += blockDim.x) smem[t] = t < 400 ? wn * gtab[kTabR + t] : -gtab[kTabR + t];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int ps = 3 * max_adj + max_padj + 1;  // plane stride: + one scratch word that idle lanes write
    // with a vertex map a fourth plane holds the vertex's pressure row (1,0)
    const int planes = fused ? 4 : 3;
    float *ring = smem + kVelTab + (size_t)w * (kVRing * kStg + ((planes * ps + 3) & ~3));
    float *acc = ring + kVRing * kStg;
    __syncthreads();
    // lane roles: (b, j) of the NA / W part for lane < 30, (i, p) = (bi, bp) of the B^T part for lane < 12
    const bool lw = lane < 30, lb = lane < 12;
    const int b = lw ? lane / 3 : 0, j = lw ? lane - 3 * (lane / 3) : 0;
    const int bi = lane >> 2, bp = lane & 3;
    const float e0 = j == 0 ? 1.0f : 0.0f, e1 = j == 1 ? 1.0f : 0.0f, e2 = j == 2 ? 1.0f : 0.0f;
    // lane-constant addresses in ring slot 0 and in the tables
    const float *pG = ring + kRecG + 12 * j;
    const float *pU = ring + kRecU + 3 * b + j;
    const float *pNA = ring + kVNA + b;
    const float *pBS = ring + kRecBS + 4 * bi;
    const float *pBSj = ring + kRecBS + 4 * j;
    const float *pP = ring + kRecP + bp;
    const uint8_t *pS = reinterpret_cast<const uint8_t *>(ring + kVSlots) + b;
    const uint8_t *pLoc = reinterpret_cast<const uint8_t *>(ring + kVSlots) + kSlotLocal;
    const uint8_t *pSp = reinterpret_cast<const uint8_t *>(ring + kVSlots) + 10 + bp;
    const float *pR = sR + 4 * b;
    const float *pY = sY + 4 * bp;
    const float *pYb = sY + 16 * b;
    // staging roles: 0 record head, 1 NA window, 2 slot map, 3 idle
    const int kind = lane < kRecVel / 4 ? 0 : (lane < kRecVel / 4 + 3 ? 1 : (lane == kRecVel / 4 + 3 ? 2 : 3));
    const int src_lane = kind == 0 ? 4 * lane : kRecNA + 4 * (lane - kRecVel / 4);
    float *dst_lane = ring + 4 * lane;
    // with `work`, nodes come from a global counter, one per warp step, so
    // all warps stay on one sharp front of the sweep and the ten readers of
    // an element's record come close in time (a fixed stride gives each warp
    // nodes of one lattice parity: vertex-heavy warps fall behind, the front
    // smears, and at 64^3 x 6 the records were read five times from DRAM)
    for (int64_t it = n_begin + (int64_t)blockIdx.x * nw + w;; it += (int64_t)gridDim.x * nw) {
        if (work) {
            unsigned long long k = 0;
            if (lane == 0) k = atomicAdd(work, 1ull);
            it = n_begin + (int64_t)__shfl_sync(0xffffffffu, k, 0);
        }
        if (it >= nnodes) break;
        const int64_t n = it;
        const int4 inf = ninfo[n];
        const int64_t i0 = node_i0(inf);
        const int m = node_m(inf);
        const IncList il = load_incidences(inc, i0, m, lane);
        const uint8_t *slots_node = slots + i0 * kSlotStride;
#pragma unroll
        for (int t = 0; t < kVRing - 1; t++)
            stage_vel<GN>(dst_lane, t, t, m, il, rec, src_lane, kind, slots_node, gstage, lane);
        const int K = node_k(inf), Kp = node_kp(inf);
        // the P1 node at this vertex, whose pressure row this warp assembles too
        const int qp = inf.z;
        for (int c = lane; c < 3 * K + Kp; c += 32) acc[c] = acc[ps + c] = acc[2 * ps + c] = 0.0f;
        if (qp >= 0)
            for (int c = lane; c < 3 * K; c += 32) acc[3 * ps + c] = 0.0f;
        float rj = 0.0f, rb = 0.0f, rq = 0.0f, rg = 0.0f;
        // the table rows of the current local index a; incidences come sorted
        // by a, so they reload only when a run of equal a ends
        int a_cur = -1;
        float4 rr = make_float4(0.f, 0.f, 0.f, 0.f), y = rr, yq = rr;
        for (int t0 = 0; t0 < m; t0 += kVRing) {
#pragma unroll
            for (int r = 0; r < kVRing; r++) {
                const int t = t0 + r;
                if (t >= m) break;
                cp_async_wait<kVRing - 2>();
                // the slot's copies are visible to the warp, and every lane is
                // done with the slot consumed in the previous step, which is
                // refilled next
                __syncwarp();
                stage_vel<GN>(dst_lane, (r + kVRing - 1) % kVRing, t + kVRing - 1, m, il, rec, src_lane, kind,
                              slots_node, gstage, lane);
                const int off = r * kStg;
                const int a = pLoc[4 * off];  // the staged slot map's local-index byte (broadcast)
                if (a != a_cur) {  // warp-uniform
                    a_cur = a;
                    rr = lds4(pR + 40 * a);
                    y = lds4(pY + 16 * a);
                    if (qp >= 0 && a < 4) yq = lds4(pYb + 4 * a);
                }
                // NA_ab on the diagonal (i = j) plus wn W_(ai)(bj), i = 0..2
                const float4 g0 = lds4(pG + off), g1 = lds4(pG + off + 4), g2 = lds4(pG + off + 8);
                const float an = pNA[off + 2 * (a & 1)];
                const int idx = lw ? 3 * pS[4 * off] + j : ps - 1;
                float *dst = acc + idx;
                // g[j][m*3+i]: m0 = (g0.x,g0.y,g0.z) m1 = (g0.w,g1.x,g1.y) m2 = (g1.z,g1.w,g2.x) m3 = (g2.y,g2.z,g2.w)
                float v0 = dst[0], v1 = dst[ps], v2 = dst[2 * ps];
                if (GN) {
                    // the viscous rows (a, i), column (b, j) = lane, and the viscous residual of row (a, lane)
                    v0 += ring[off + kVGn + lane];
                    v1 += ring[off + kVGn + 32 + lane];
                    v2 += ring[off + kVGn + 64 + lane];
                    rg += ring[off + kVGnRes + ((3 * a) & 3) + (lane & 3)];
                }
                dst[0] = fmaf(g2.y, rr.w, fmaf(g1.z, rr.z, fmaf(g0.w, rr.y, fmaf(g0.x, rr.x, fmaf(e0, an, v0)))));
                dst[ps] = fmaf(g2.z, rr.w, fmaf(g1.w, rr.z, fmaf(g1.x, rr.y, fmaf(g0.y, rr.x, fmaf(e1, an, v1)))));
                dst[2 * ps] = fmaf(g2.w, rr.w, fmaf(g2.x, rr.z, fmaf(g1.y, rr.y, fmaf(g0.z, rr.x, fmaf(e2, an, v2)))));
                const float ub = pU[off];
                rj = fmaf(an, ub, rj);
                // -Bd_p(a, i): the (0,1) entry of velocity row (a, i), pressure column p
                const float4 bs = lds4(pBS + off);
                const float bt = fmaf(bs.z, y.z, fmaf(bs.y, y.y, bs.x * y.x));
                float *dp = acc + (lb ? bi * ps + 3 * K + pSp[4 * off] : ps - 1);
                *dp += bt;
                rb = fmaf(bt, pP[off], rb);
                if (qp >= 0 && a < 4) {
                    // -Bd_q(b j): the (1,0) entry of pressure row q = this vertex, column (b, j)
                    const float4 bj = lds4(pBSj + off);
                    const float pv = fmaf(bj.z, yq.z, fmaf(bj.y, yq.y, bj.x * yq.x));
                    acc[3 * ps + idx] += pv;
                    rq = fmaf(pv, ub, rq);
                }
            }
        }
        cp_async_wait<0>();
        __syncwarp();
        if (vals00) {
            double *out = vals00 + rowptr00[3 * n];
            for (int c = lane; c < 3 * K; c += 32) {
                st_cs(out + c, f2d_exact(acc[c]));
                st_cs(out + 3 * K + c, f2d_exact(acc[ps + c]));
                st_cs(out + 6 * K + c, f2d_exact(acc[2 * ps + c]));
            }
            double *out1 = vals01 + rowptr01[3 * n];
            const float *accp = acc + 3 * K;
            for (int c = lane; c < Kp; c += 32) {
                st_cs(out1 + c, f2d_exact(accp[c]));
                st_cs(out1 + Kp + c, f2d_exact(accp[ps + c]));
                st_cs(out1 + 2 * Kp + c, f2d_exact(accp[2 * ps + c]));
            }
        }
        if (res_u) {
            // row (a, i) sums rj over the lanes 3 b + i and rb over the lanes
            // 4 i + p: strided tree sums leave them in lanes i = 0..2 and 4 i
            float x = lw ? rj : 0.0f, z = lb ? rb : 0.0f;
#pragma unroll
            for (int d = 3; d < 32; d *= 2) {
                const float y = __shfl_down_sync(0xffffffffu, x, d);
                if (lane + d < 32) x += y;
            }
#pragma unroll
            for (int d = 1; d < 4; d *= 2) {
                const float y = __shfl_down_sync(0xffffffffu, z, d);
                if (lane + d < 32) z += y;
            }
            z = __shfl_sync(0xffffffffu, z, lane < 3 ? 4 * lane : 0);
            // uu (N(u) u + viscous) + up (-B^T p), with the residual's block factors
            const float cuu = (float)co.uu, s = fmaf(cuu, x, (float)co.up * z);
            if (lane < 3) res_u[3 * n + lane] = f2d_exact(GN ? fmaf(cuu, rg, s) : s);
        }
        if (qp >= 0) {
            if (vals10) {
                double *out = vals10 + rowptr10[qp];
                for (int c = lane; c < 3 * K; c += 32) st_cs(out + c, f2d_exact(acc[3 * ps + c]));
            }
            if (res_p) {
                const float v = warp_sum(lw ? rq : 0.0f);
                if (lane == 0) res_p[qp] = f2d_exact((float)co.pu * v);
            }
        }
        __syncwarp();
    }
}

// pressure rows: block (1,0) values and the pressure residual.  One warp per
// pressure node q; per incidence lanes 0-10 copy the record's Bs and u
// (floats [kRecBS, kRecBS + 44)) and lane 11 the slot map into a ring slot
// with one 16-byte cp.async each; lane (b, d) < 30 adds -Bd_q(b d).
constexpr int kPRing = 4;
constexpr int kPStage = 48;  // floats per ring slot: Bs 12 | u 30 | pad 2 | slot map 16 B
constexpr int kPU = kRecU - kRecBS, kPSlots = 44;
static_assert(kRecU == kRecBS + 12 && kRecP <= kRecBS + kPSlots, "Bs and u are adjacent in the record");

__device__ __forceinline__ void stage_pres(float *dst_lane, int slot, int t, int m, const IncList &il,
                                           const float *__restrict__ rec_lane, int lane,
                                           const uint8_t *__restrict__ slots_node) {
    if (t < m) {
        const uint32_t ea = incidence_at(il, t);
        const void *src = lane == kPSlots / 4 ? static_cast<const void *>(slots_node + t * kSlotStride)
                                              : static_cast<const void *>(rec_lane + (size_t)(ea >> 4) * kNSRecord);
        if (lane <= kPSlots / 4) cp_async16(dst_lane + slot * kPStage, src);
    }
    cp_async_commit();
}

__global__ void __launch_bounds__(256) k_ns_pres_rows(const int64_t *__restrict__ inc_ptr, const uint32_t *__restrict__ inc,
                                                      const uint8_t *__restrict__ slots, const int64_t *__restrict__ adj_ptr,
                                                      const float *__restrict__ rec, const float *__restrict__ gtab,
                                                      const int64_t *__restrict__ rowptr10, double *vals10, double *res_p,
                                                      int64_t nnodes, int max_adj, float cpu) {
    extern __shared__ __align__(16) float smem[];
    float *sY = smem;  // -Y[b][q][4]
    for (int t = threadIdx.x; t < 160; t += blockDim.x) sY[t] = -gtab[kTabY + t];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int acc_words = (3 * max_adj + 1 + 3) & ~3;  // + one scratch word that idle lanes write
    float *ring = smem + 160 + (size_t)w * (kPRing * kPStage + acc_words);
    float *acc = ring + kPRing * kPStage;
    const bool lw = lane < 30;
    const int b = lw ? lane / 3 : 0, d = lw ? lane - 3 * (lane / 3) : 0;
    const float *pBS = ring + 4 * d;
    const float *pU = ring + kPU + 3 * b + d;
    const uint8_t *pS = reinterpret_cast<const uint8_t *>(ring + kPSlots) + b;
    const float *pY = sY + 16 * b;
    float *dst_lane = ring + 4 * lane;
    const float *rec_lane = rec + kRecBS + 4 * lane;
    for (int64_t n = (int64_t)blockIdx.x * nw + w; n < nnodes; n += (int64_t)gridDim.x * nw) {
        const int64_t i0 = inc_ptr[n], i1 = inc_ptr[n + 1];
        const int m = (int)(i1 - i0);
        const IncList il = load_incidences(inc, i0, m, lane);
        const uint8_t *slots_node = slots + i0 * kSlotStride;
#pragma unroll
        for (int t = 0; t < kPRing - 1; t++) stage_pres(dst_lane, t, t, m, il, rec_lane, lane, slots_node);
        const int K = (int)(adj_ptr[n + 1] - adj_ptr[n]);
        for (int c = lane; c < 3 * K; c += 32) acc[c] = 0.0f;
        float r = 0.0f;
        for (int t0 = 0; t0 < m; t0 += kPRing) {
#pragma unroll
            for (int rs = 0; rs < kPRing; rs++) {
                const int t = t0 + rs;
                if (t >= m) break;
                cp_async_wait<kPRing - 2>();
                __syncwarp();
                stage_pres(dst_lane, (rs + kPRing - 1) % kPRing, t + kPRing - 1, m, il, rec_lane, lane, slots_node);
                const int off = rs * kPStage;
                const int q = (int)(incidence_at(il, t) & 15u);
                const float4 bs = lds4(pBS + off);
                const float4 y = lds4(pY + 4 * q);
                const float v = fmaf(bs.z, y.z, fmaf(bs.y, y.y, bs.x * y.x));
                float *dst = acc + (lw ? 3 * pS[4 * off] + d : 3 * max_adj);
                *dst += v;
                r = fmaf(v, pU[off], r);
            }
        }
        cp_async_wait<0>();
        __syncwarp();
        if (vals10) {
            double *out = vals10 + rowptr10[n];
            for (int c = lane; c < 3 * K; c += 32) st_cs(out + c, f2d_exact(acc[c]));
        }
        if (res_p) {
            float v = warp_sum(lw ? r : 0.0f);
            if (lane == 0) res_p[n] = f2d_exact(cpu * v);
        }
        __syncwarp();
    }
}

// dense 34x34 element matrices and element residuals (AssembleFE view)
__global__ void k_ns_dense(const float *__restrict__ rec, const float *__restrict__ gtab, int64_t first, int64_t count,
                           float visc_dens, float dens, int newton, double *Ke, double *re, NSCoeff co) {
    const int64_t e = blockIdx.x;
    if (e >= count) return;
    const int lane = threadIdx.x;
    const float *R = rec + (first + e) * kNSRecord;
    double *J = Ke + e * 34 * 34;
    double *r = re + e * 34;
    for (int t = lane; t < 34 * 34; t += 32) J[t] = 0.0;
    __syncwarp();
    const int b = lane < 30 ? lane / 3 : 0, j = lane < 30 ? lane % 3 : 0;
    float rr[3] = {0, 0, 0};
    for (int a = 0; a < 10; a++) {
        float wv[3] = {0, 0, 0}, part = 0.0f;
        if (lane < 30) part = ns_lane_terms(R, gtab, a, b, j, visc_dens, dens, wv);
        float an = sum3_lanes(part, lane);
        float racc = 0.0f;
        if (lane < 30) {
            for (int i = 0; i < 3; i++) {
                float v = (i == j ? an : 0.0f);
                if (newton) v = fmaf(dens, wv[i], v);
                J[(3 * a + i) * 34 + 3 * b + j] = (double)v;
            }
            racc = an * R[kRecU + 3 * b + j];
        }
        for (int i = 0; i < 3; i++) {
            float s = warp_sum((lane < 30 && j == i) ? racc : 0.0f);
            if (lane == 0) rr[i] = s;
        }
        if (lane < 12) {
            int bi = lane >> 2, bp = lane & 3;
            float v = ns_bt(R, gtab, a, bi, bp);
            J[(3 * a + bi) * 34 + 30 + bp] = (double)v;
            J[(30 + bp) * 34 + 3 * a + bi] = (double)v;
        }
        __syncwarp();
        if (lane == 0) {
            for (int i = 0; i < 3; i++) {
                double s = co.uu * (double)rr[i];
                for (int pp = 0; pp < 4; pp++) s = fma(co.up * J[(3 * a + i) * 34 + 30 + pp], (double)R[kRecP + pp], s);
                r[3 * a + i] = s;
            }
        }
        __syncwarp();
    }
    if (lane < 4) {
        double s = 0.0;
        for (int k = 0; k < 30; k++) s += J[(30 + lane) * 34 + k] * (double)R[kRecU + k];
        r[30 + lane] = co.pu * s;
    }
}

int sm_count_ns() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

void ns_upload_tables(const NSTables &t, float **d_tables) {
    std::vector<float> h(kTabSize, 0.0f);
    for (int c = 0; c < 3; c++)
        for (int a = 0; a < 10; a++)
            for (int b = 0; b < 10; b++)
                for (int k = 0; k < 10; k++) h[kTabT + ((a * 3 + k / 4) * 32 + 3 * b + c) * 4 + k % 4] = t.T[c][a][b][k];
    for (int a = 0; a < 10; a++)
        for (int b = 0; b < 10; b++) {
            for (int s = 0; s < 6; s++) h[kTabKS + (a * 10 + b) * 6 + s] = t.KS[a][b][s];
            for (int m = 0; m < 4; m++) h[kTabR + (a * 10 + b) * 4 + m] = t.R[a][b][m];
        }
    for (int b = 0; b < 10; b++)
        for (int p = 0; p < 4; p++)
            for (int c = 0; c < 3; c++) h[kTabY + (b * 4 + p) * 4 + c] = t.Y[c][p][b];
    FEDD_CUDA(cudaMalloc(d_tables, kTabSize * sizeof(float)));
    FEDD_CUDA(cudaMemcpy(*d_tables, h.data(), kTabSize * sizeof(float), cudaMemcpyHostToDevice));
    FEDD_CUDA(cudaMemcpyToSymbol(c_dv, t.DV, sizeof t.DV));


}

void launch_ns_record(const double *xyz, const int32_t *conn2, const int32_t *conn1, int64_t ne, const double *u,
                      const double *p, const float *d_tables, float visc_dens, float dens, float *rec, int *d_err,
                      cudaStream_t s, LaunchCounter &lc, int64_t e_begin, int64_t e_end) {
    if (e_end < 0) e_end = ne;
    const int64_t count = e_end - e_begin;
    if (count <= 0) return;
    // persistent CTAs, one per SM (shared memory, all 512 TMEM columns)
    const unsigned grid = (unsigned)std::min<int64_t>(ceil_div(count, (int64_t)kRecTile * kRecGroups), (int64_t)sm_count_ns());
    FEDD_CUDA(cudaFuncSetAttribute(k_ns_record, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRecSmem));
    k_ns_record<<<grid, kRecThreads, kRecSmem, s>>>(xyz, conn2, conn1, ne, u, p, rec, d_err, e_begin, e_end, d_tables,
                                                  visc_dens, dens);
    FEDD_CUDA(cudaGetLastError());
    lc.n += 1;
}

void launch_ns_node_info(const Graph &g, const int64_t *padj_ptr, const int32_t *vmap, int4 *info, cudaStream_t s) {
    const int64_t nn = g.nrow_nodes;
    if (nn == 0) return;
    k_ns_node_info<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(g.inc_ptr.p, g.adj_ptr.p, padj_ptr, vmap, nn, info);
    FEDD_CUDA(cudaGetLastError());
}

void launch_ns_vel_rows(const Graph &g, const int4 *ninfo, const float *rec, const float *d_tables,
                        const int64_t *rowptr00, const int64_t *rowptr01, double *vals00, double *vals01, double *res_u,
                        float visc_dens, float dens, int newton, int want_jac, int max_adj, int max_padj,
                        const int32_t *vmap, const int64_t *rowptr10, double *vals10, double *res_p,
                        const float *gstage, cudaStream_t s, LaunchCounter &lc, int64_t n_begin, int64_t n_end,
                        unsigned long long *work, const NSCoeff &co) {
    (void)visc_dens;  // nu rho enters through NA, which the record kernels wrote
    // up to 16 warps share one copy of the tables; two CTAs fit an SM at the
    // structured meshes' adjacency, fewer warps where the accumulators are larger
    const bool gn = gstage != nullptr;
    const int planes = vmap ? 4 : 3;
    const int acc_words = (planes * (3 * max_adj + max_padj + 1) + 3) & ~3;
    const size_t per_warp = (size_t)(kVRing * (gn ? kVStageGn : kVStage) + acc_words) * sizeof(float);
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(16, (227 * 1024 - kVelTab * sizeof(float)) / per_warp));
    size_t smem = kVelTab * sizeof(float) + (size_t)warps * per_warp;
    auto kern = gn ? k_ns_vel_rows<true> : k_ns_vel_rows<false>;
    FEDD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t nn = n_end < 0 ? g.nrow_nodes : n_end;
    unsigned grid = (unsigned)std::min<int64_t>((nn - n_begin + warps - 1) / warps, (int64_t)sm_count_ns() * 4);
    if (work) {  // dynamic positions: exactly the CTAs that fit
        int per_sm = 0;
        FEDD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * warps, smem));
        grid = (unsigned)std::min<int64_t>(grid, (int64_t)sm_count_ns() * std::max(per_sm, 1));
        FEDD_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned long long), s));
    }
    if (grid == 0) return;
    kern<<<grid, 32 * warps, smem, s>>>(ninfo, g.inc.p, g.slots.p, rec, d_tables, rowptr00, rowptr01,
                                        want_jac ? vals00 : nullptr, want_jac ? vals01 : nullptr, res_u, nn, dens,
                                        newton, max_adj, max_padj, n_begin, vmap ? 1 : 0, rowptr10,
                                        want_jac ? vals10 : nullptr, res_p, gstage, work, co);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

void launch_ns_pres_rows(const Graph &gp, const float *rec, const float *d_tables, const int64_t *rowptr10,
                         double *vals10, double *res_p, int want_jac, int max_adj, cudaStream_t s, LaunchCounter &lc,
                         const NSCoeff &co) {
    const int warps = 8;
    const int acc_words = (3 * max_adj + 1 + 3) & ~3;
    size_t smem = (160 + (size_t)warps * (kPRing * kPStage + acc_words)) * sizeof(float);
    FEDD_CUDA(cudaFuncSetAttribute(k_ns_pres_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t nn = gp.nrow_nodes;
    unsigned grid = (unsigned)std::min<int64_t>((nn + warps - 1) / warps, (int64_t)sm_count_ns() * 8);
    if (grid == 0) return;
    k_ns_pres_rows<<<grid, 32 * warps, smem, s>>>(gp.inc_ptr.p, gp.inc.p, gp.slots.p, gp.adj_ptr.p, rec, d_tables,
                                                  rowptr10, want_jac ? vals10 : nullptr, res_p, nn, max_adj,
                                                  (float)co.pu);
    FEDD_CUDA(cudaGetLastError());
    lc.n++;
}

void launch_ns_dense(const float *rec, const float *d_tables, int64_t first, int64_t count, float visc_dens,
                     float dens, int newton, double *Ke, double *re, cudaStream_t s, const NSCoeff &co) {
    if (count == 0) return;
    k_ns_dense<<<(unsigned)count, 32, 0, s>>>(rec, d_tables, first, count, visc_dens, dens, newton, Ke, re, co);
    FEDD_CUDA(cudaGetLastError());
}

}  // namespace fedd
