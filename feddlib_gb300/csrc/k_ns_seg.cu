// k_ns_seg.cu -- Navier-Stokes rows as segmented reductions over each row's
// column slots.
//
// The rows of FE::assemblyNavierStokes (feddlib/core/FE/FE_def.hpp:1153-1213
// element loop, addFeBlockMatrix :982-1062, residual export :1223-1236): every
// CSR value of velocity row (n, i) is the sum over the elements t containing
// node n and column node c of the element block (a_t, b_t), where a_t and b_t
// are the local indices of n and c in t.  For a row node n with K column
// nodes (slots) and m incidences there are 10 m such (t, b) contributions.
//
// Graph build (once per mesh) sorts each row node's contributions by slot,
// then by incidence, into 16-bit codes, and cuts the row nodes into batches
// of consecutive nodes with at most BI incidences.  Per batch a warp stages
// the incidences' record data (velocity gradients at the vertices g, Bs, u,
// p and the row's NA entries) transposed, one float row per quantity with an
// odd stride, so that lanes reading the same quantity of different
// incidences never share a bank.  Each lane then takes a contiguous chunk of
// the batch's slot-sorted contributions and sums the ones of a slot in
// registers: for contribution (t, b) of row node a
//   W_(ai)(bj) = wn sum_m g_t[j][m][i] R[a][b][m]      (Newton term, wn = rho or 0)
//   + NA_t[a][b] on i = j                               (nu rho A + rho N)
//   bt_i = -sum_c Bs_t[i][c] Y[c][b][a]   (b < 4)       (block (0,1), column P1 node b)
//   pv_j = -sum_c Bs_t[j][c] Y[c][a][b]   (a < 4)       (block (1,0), row = vertex a)
// A slot split between neighbouring lanes is combined left to right by
// shuffles, so every value is the sum of its contributions in one fixed
// order (deterministic, no atomics, no read-modify-write of shared
// accumulators).  The slots' sums go to per-slot records in shared memory;
// the batch's rows are written out from them once, FP32 converted exactly to
// FP64, with the residuals r_u = sum_s (NAsum_s u_s + bt_s p_s) and
// r_p = sum_s pv_s . u_s.
//
// Block (0,1) comes from the vertex columns of the velocity row: with
// Taylor-Hood the row's P1 columns are the P1 nodes of its P2 vertex
// columns, in the same order when the vertex map is monotone on every row
// (verified at graph build, else the engine keeps the incidence-ring kernel
// of k_ns.cu).
#include "kernels.cuh"

namespace fedd {
namespace {

// table layout (must match k_ns.cu)
constexpr int kTabR = 4440;   // R[a][b][4]
constexpr int kTabY = 4840;   // Y[b][p][4]: Y[c][p][b] at kTabY + (b * 4 + p) * 4 + c
// record layout (must match k_ns.cu)
constexpr int kRecG = 0, kRecBS = 36, kRecU = 48, kRecP = 78, kRecNA = 128;

// staged rows per incidence (each a row of S floats, S odd)
constexpr int kSG = 0;     // g[f], f = 12 j + 3 m + i          36
constexpr int kSBs = 36;   // Bs[i][c] at 36 + 3 i + c          9
constexpr int kSU = 45;    // u[b][i] at 45 + 3 b + i           30
constexpr int kSP = 75;    // p[0..3]                           4
constexpr int kSNA = 79;   // NA[a][b] at 79 + b                10
constexpr int kSA = 89;    // local index a of the row node     1
constexpr int kStgRows = 90;

// per-slot record: W+NA block (3 i + j) | NAsum | (bt_i, pv_i) pairs | code | pad
constexpr int kSegRec = 18;
constexpr int kRecNas = 9, kRecBt = 10, kRecCode = 16;

constexpr uint32_t kCodeSeg = 0x8000u, kCodeRow = 0x4000u;

constexpr int kTabStride = 101;           // [10 quantities][100 (a, b)] + 1
constexpr int kTabFloats = 10 * kTabStride + 2;

template <int BI, int BS> struct SegCfg {
    static constexpr int S = BI + 1;                             // odd
    static constexpr int CMAX = 2 * ((10 * BI + 63) / 64);       // codes per lane (even)
    static constexpr int kStage = kStgRows * S;
    static constexpr int kRecs = BS * kSegRec;
    static constexpr int kPslot = (BS + 3) / 4;                  // int8 per slot, as words
    static constexpr int kPerWarp = (kStage + kRecs + kPslot + 3) & ~3;
};

__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    unsigned long long ra = *reinterpret_cast<unsigned long long *>(&a);
    unsigned long long rb = *reinterpret_cast<unsigned long long *>(&b);
    unsigned long long rc = *reinterpret_cast<unsigned long long *>(&c);
    unsigned long long rd;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
    return *reinterpret_cast<float2 *>(&rd);
}

struct SegArgs {
    const int32_t *batch_node;   // nb + 1 node boundaries
    const uint16_t *codes;       // 10 per incidence, node order
    const int8_t *pslot;         // per adjacency entry: position among the row's P1 columns, -1 for edge nodes
    const int64_t *inc_ptr;
    const uint32_t *inc;
    const int64_t *adj_ptr, *padj_ptr;
    const int32_t *vmap;
    const float *rec, *gtab;
    const int64_t *rowptr00, *rowptr01, *rowptr10;
    double *vals00, *vals01, *vals10, *res_u, *res_p;
    float dens;
    int newton;
    int64_t b_begin, b_end;
    unsigned long long *work;
};

// one contribution (t, b) of the row node with local index a into acc
// acc: w[0..8] (3 i + j), nas, (bt0, pv0), (bt1, pv1), (bt2, pv2)
template <int S>
__device__ __forceinline__ void seg_contribution(float *acc, const float *__restrict__ stg,
                                                 const float *__restrict__ tab, uint32_t code) {
    const int t = (int)((code >> 4) & 63u), b = (int)(code & 15u);
    const float *G = stg + t;
    const int a = __float_as_int(G[kSA * S]);
    const int ab = 10 * a + b;
    const float r0 = tab[ab], r1 = tab[kTabStride + ab], r2 = tab[2 * kTabStride + ab], r3 = tab[3 * kTabStride + ab];
    const float2 q0 = make_float2(r0, r0), q1 = make_float2(r1, r1), q2 = make_float2(r2, r2), q3 = make_float2(r3, r3);
    // W(i, j) = sum_m g[12 j + 3 m + i] r_m, outputs o = 3 i + j in pairs (0,1) (2,3) (4,5) (6,7) and o = 8
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const int o0 = 2 * p, o1 = 2 * p + 1;
        const int f0 = 12 * (o0 % 3) + o0 / 3, f1 = 12 * (o1 % 3) + o1 / 3;
        float2 s = make_float2(acc[o0], acc[o1]);
        s = ffma2(make_float2(G[(kSG + f0) * S], G[(kSG + f1) * S]), q0, s);
        s = ffma2(make_float2(G[(kSG + f0 + 3) * S], G[(kSG + f1 + 3) * S]), q1, s);
        s = ffma2(make_float2(G[(kSG + f0 + 6) * S], G[(kSG + f1 + 6) * S]), q2, s);
        s = ffma2(make_float2(G[(kSG + f0 + 9) * S], G[(kSG + f1 + 9) * S]), q3, s);
        acc[o0] = s.x;
        acc[o1] = s.y;
    }
    {   // o = 8: i = j = 2, f = 26
        float s = acc[8];
        s = fmaf(G[(kSG + 26) * S], r0, s);
        s = fmaf(G[(kSG + 29) * S], r1, s);
        s = fmaf(G[(kSG + 32) * S], r2, s);
        s = fmaf(G[(kSG + 35) * S], r3, s);
        acc[8] = s;
    }
    const float na = G[(kSNA + b) * S];
    acc[0] += na;
    acc[4] += na;
    acc[8] += na;
    acc[9] += na;
    const float ya0 = tab[4 * kTabStride + ab], ya1 = tab[5 * kTabStride + ab], ya2 = tab[6 * kTabStride + ab];
    const float yb0 = tab[7 * kTabStride + ab], yb1 = tab[8 * kTabStride + ab], yb2 = tab[9 * kTabStride + ab];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float s0 = G[(kSBs + 3 * i) * S], s1 = G[(kSBs + 3 * i + 1) * S], s2 = G[(kSBs + 3 * i + 2) * S];
        acc[10 + 2 * i] = fmaf(s2, ya2, fmaf(s1, ya1, fmaf(s0, ya0, acc[10 + 2 * i])));
        acc[11 + 2 * i] = fmaf(s2, yb2, fmaf(s1, yb1, fmaf(s0, yb0, acc[11 + 2 * i])));
    }
}

__device__ __forceinline__ void seg_flush(float *recs, int seg, const float *acc, uint32_t code) {
    float2 *R = reinterpret_cast<float2 *>(recs + seg * kSegRec);
#pragma unroll
    for (int k = 0; k < 8; k++) R[k] = make_float2(acc[2 * k], acc[2 * k + 1]);
    R[8] = make_float2(__uint_as_float(code), 0.0f);
}

template <int BI, int BS>
__global__ void __launch_bounds__(32 * 12) k_ns_seg_rows(const SegArgs A) {
    using C = SegCfg<BI, BS>;
    constexpr int S = C::S, CMAX = C::CMAX;
    extern __shared__ __align__(16) float smem[];
    float *tab = smem;
    const float wn = A.newton ? A.dens : 0.0f;
    for (int x = threadIdx.x; x < 1000; x += blockDim.x) {
        const int k = x / 100, ab = x - 100 * k, a = ab / 10, b = ab - 10 * a;
        float v;
        if (k < 4) v = wn * A.gtab[kTabR + ab * 4 + k];
        else if (k < 7) v = b < 4 ? -A.gtab[kTabY + (a * 4 + b) * 4 + (k - 4)] : 0.0f;
        else v = a < 4 ? -A.gtab[kTabY + (b * 4 + a) * 4 + (k - 7)] : 0.0f;
        tab[k * kTabStride + ab] = v;
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *stg = smem + kTabFloats + (size_t)w * C::kPerWarp;
    float *recs = stg + C::kStage;
    int8_t *ps_s = reinterpret_cast<int8_t *>(recs + C::kRecs);
    __syncthreads();
    // staging roles: lane copies staged rows k = lane + 32 q (q < 3, k < 89) from record offset src[q]
    int src[3];
    bool na_row[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int k = lane + 32 * q;
        int o = -1;
        if (k < kSBs) o = kRecG + k;
        else if (k < kSU) o = kRecBS + 4 * ((k - kSBs) / 3) + (k - kSBs) % 3;
        else if (k < kSNA) o = kRecU + (k - kSU);      // u then p: kRecP = kRecU + 30
        else if (k < kSA) o = kRecNA + (k - kSNA);     // + 10 a per incidence
        src[q] = o;
        na_row[q] = k >= kSNA && k < kSA;
    }
    static_assert(kRecP == kRecU + 30 && kSP == kSU + 30, "u and p adjacent in record and stage");

    for (;;) {
        int64_t bi;
        {
            unsigned long long k = 0;
            if (lane == 0) k = atomicAdd(A.work, 1ull);
            bi = A.b_begin + (int64_t)__shfl_sync(0xffffffffu, k, 0);
        }
        if (bi >= A.b_end) break;
        const int n0 = A.batch_node[bi], n1 = A.batch_node[bi + 1];
        const int nr = n1 - n0;
        const int64_t i0 = A.inc_ptr[n0];
        const int mb = (int)(A.inc_ptr[n1] - i0);
        const int64_t sb0 = A.adj_ptr[n0];
        const int nseg = (int)(A.adj_ptr[n1] - sb0);
        // rows of the batch, one per lane
        int rK = 0, rKp = 0, rq = -1, rs = nseg;
        if (lane < nr) {
            const int n = n0 + lane;
            const int64_t a0 = A.adj_ptr[n];
            rK = (int)(A.adj_ptr[n + 1] - a0);
            rKp = (int)(A.padj_ptr[n + 1] - A.padj_ptr[n]);
            rq = A.vmap[n];
            rs = (int)(a0 - sb0);
        }
        // stage the incidences (4-byte copies into the transposed rows)
        const uint32_t incv = lane < mb ? __ldg(A.inc + i0 + lane) : 0u;
        for (int t = 0; t < mb; t++) {
            const uint32_t v = __shfl_sync(0xffffffffu, incv, t);
            const float *r = A.rec + (size_t)(v >> 4) * kNSRecord;
            const int a = (int)(v & 15u);
#pragma unroll
            for (int q = 0; q < 3; q++)
                if (src[q] >= 0) cp_async4(stg + (lane + 32 * q) * S + t, r + src[q] + (na_row[q] ? 10 * a : 0));
            if (lane == 0) stg[kSA * S + t] = __int_as_float(a);
        }
        cp_async_commit();
        for (int x = lane; x < nseg; x += 32) ps_s[x] = A.pslot[sb0 + x];
        // this lane's chunk of the batch's contributions
        const int Ctot = 10 * mb;
        const int c = 2 * ((Ctot + 63) / 64);
        const int k0 = lane * c;
        const int nmine = max(0, min(c, Ctot - k0));
        uint32_t cw[CMAX / 2];
        const uint32_t *cp = reinterpret_cast<const uint32_t *>(A.codes + 10 * i0 + k0);
#pragma unroll
        for (int q = 0; q < CMAX / 2; q++) cw[q] = 2 * q < nmine ? __ldg(cp + q) : 0u;
        int nflags = 0;
#pragma unroll
        for (int q = 0; q < CMAX; q++)
            if (q < nmine) nflags += (cw[q >> 1] >> (16 * (q & 1))) & kCodeSeg ? 1 : 0;
        int before = nflags;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, before, o);
            if (lane >= o) before += y;
        }
        before -= nflags;
        const bool first_start = nmine > 0 && (cw[0] & kCodeSeg);
        const bool open_left = nmine > 0 && !first_start;
        int seg = before - (first_start ? 0 : 1);
        cp_async_wait<0>();
        __syncwarp();

        float acc[16], lp[16];
#pragma unroll
        for (int x = 0; x < 16; x++) acc[x] = lp[x] = 0.0f;
        bool first = true;
        uint32_t last = 0;
#pragma unroll
        for (int q = 0; q < CMAX; q++) {
            if (q < nmine) {
                const uint32_t code = (cw[q >> 1] >> (16 * (q & 1))) & 0xffffu;
                if (q > 0 && (code & kCodeSeg)) {
                    if (first && open_left) {
#pragma unroll
                        for (int x = 0; x < 16; x++) lp[x] = acc[x];
                    } else {
                        seg_flush(recs, seg, acc, last);
                    }
                    first = false;
#pragma unroll
                    for (int x = 0; x < 16; x++) acc[x] = 0.0f;
                    seg++;
                }
                seg_contribution<S>(acc, stg, tab, code);
                last = code;
            }
        }
        // slots split between lanes: the lane holding a slot's first piece
        // adds the pieces of the following lanes, left to right
        const bool single = nmine > 0 && first;
        const bool next_open = __shfl_down_sync(0xffffffffu, open_left ? 1 : 0, 1) && lane < 31;
        if (single && open_left) {
#pragma unroll
            for (int x = 0; x < 16; x++) lp[x] = acc[x];
        }
        const bool middle = single && open_left && next_open;
        const bool holder = nmine > 0 && !(single && open_left);
        bool active = holder && next_open;
        for (int d = 1; d < 32; d++) {
            if (!__any_sync(0xffffffffu, active)) break;
            const bool mid_d = __shfl_down_sync(0xffffffffu, middle ? 1 : 0, d);
#pragma unroll
            for (int x = 0; x < 16; x++) {
                const float v = __shfl_down_sync(0xffffffffu, lp[x], d);
                if (active) acc[x] += v;
            }
            active = active && mid_d;
        }
        if (holder) seg_flush(recs, seg, acc, last);
        __syncwarp();

        // write-out, row by row
        for (int r = 0; r < nr; r++) {
            const int n = n0 + r;
            const int K = __shfl_sync(0xffffffffu, rK, r), Kp = __shfl_sync(0xffffffffu, rKp, r);
            const int q = __shfl_sync(0xffffffffu, rq, r), sb = __shfl_sync(0xffffffffu, rs, r);
            const float *RS = recs + sb * kSegRec;
            if (A.vals00) {
                double *out = A.vals00 + A.rowptr00[3 * (int64_t)n];
#pragma unroll
                for (int i = 0; i < 3; i++)
                    for (int x = lane; x < 3 * K; x += 32) {
                        const int s = x / 3, j = x - 3 * s;
                        st_cs(out + i * 3 * K + x, f2d_exact(RS[s * kSegRec + 3 * i + j]));
                    }
                double *o1 = A.vals01 + A.rowptr01[3 * (int64_t)n];
                for (int s = lane; s < K; s += 32) {
                    const int ps = ps_s[sb + s];
                    if (ps >= 0) {
#pragma unroll
                        for (int i = 0; i < 3; i++) st_cs(o1 + i * Kp + ps, f2d_exact(RS[s * kSegRec + kRecBt + 2 * i]));
                    }
                }
                if (q >= 0) {
                    double *o2 = A.vals10 + A.rowptr10[q];
                    for (int x = lane; x < 3 * K; x += 32) {
                        const int s = x / 3, j = x - 3 * s;
                        st_cs(o2 + x, f2d_exact(RS[s * kSegRec + kRecBt + 1 + 2 * j]));
                    }
                }
            }
            if (A.res_u) {
                float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, rp = 0.0f;
                for (int s = lane; s < K; s += 32) {
                    const float *R = RS + s * kSegRec;
                    const uint32_t code = __float_as_uint(R[kRecCode]);
                    const int t = (int)((code >> 4) & 63u), b = (int)(code & 15u);
                    const float u0 = stg[(kSU + 3 * b) * S + t], u1 = stg[(kSU + 3 * b + 1) * S + t],
                                u2 = stg[(kSU + 3 * b + 2) * S + t];
                    const float pc = b < 4 ? stg[(kSP + b) * S + t] : 0.0f;
                    const float nas = R[kRecNas];
                    r0 = fmaf(R[kRecBt], pc, fmaf(nas, u0, r0));
                    r1 = fmaf(R[kRecBt + 2], pc, fmaf(nas, u1, r1));
                    r2 = fmaf(R[kRecBt + 4], pc, fmaf(nas, u2, r2));
                    rp = fmaf(R[kRecBt + 5], u2, fmaf(R[kRecBt + 3], u1, fmaf(R[kRecBt + 1], u0, rp)));
                }
                r0 = warp_sum(r0);
                r1 = warp_sum(r1);
                r2 = warp_sum(r2);
                rp = warp_sum(rp);
                if (lane == 0) {
                    A.res_u[3 * (int64_t)n] = f2d_exact(r0);
                    A.res_u[3 * (int64_t)n + 1] = f2d_exact(r1);
                    A.res_u[3 * (int64_t)n + 2] = f2d_exact(r2);
                    if (q >= 0 && A.res_p) A.res_p[q] = f2d_exact(rp);
                }
            }
        }
        __syncwarp();
    }
}

// ---- graph build ---------------------------------------------------------
// pslot of every adjacency entry of every velocity row node, and the check
// that the row's P1 columns are exactly its P2 vertex columns mapped through
// vmap, in the same order
__global__ void k_seg_pslot(int64_t nn, const int64_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj,
                            const int64_t *__restrict__ padj_ptr, const int32_t *__restrict__ padj,
                            const int32_t *__restrict__ vmap, int8_t *pslot, int *bad) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int64_t p0 = padj_ptr[n], p1 = padj_ptr[n + 1];
    if (p1 - p0 > 127) {
        atomicExch(bad, 1);
        return;
    }
    int64_t j = p0;
    for (int64_t x = adj_ptr[n]; x < adj_ptr[n + 1]; x++) {
        const int32_t v = vmap[adj[x]];
        if (v >= 0) {
            if (j >= p1 || padj[j] != v) {
                atomicExch(bad, 1);
                return;
            }
            pslot[x] = (int8_t)(j - p0);
            j++;
        } else {
            pslot[x] = -1;
        }
    }
    if (j != p1) atomicExch(bad, 1);
}

// the slot-sorted contribution codes of every batch: b | t << 4 (t relative
// to the batch's first incidence), kCodeSeg on a slot's first contribution,
// kCodeRow on a row node's first
__global__ void k_seg_codes(const int32_t *__restrict__ batch_node, int64_t nb, const int64_t *__restrict__ inc_ptr,
                            const uint8_t *__restrict__ slots, const int64_t *__restrict__ adj_ptr, uint16_t *codes) {
    const int64_t bi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (bi >= nb) return;
    const int n0 = batch_node[bi], n1 = batch_node[bi + 1];
    const int64_t i0 = inc_ptr[n0];
    uint16_t cnt[kMaxAdjacency + 1];
    for (int n = n0; n < n1; n++) {
        const int64_t ib = inc_ptr[n], ie = inc_ptr[n + 1];
        const int K = (int)(adj_ptr[n + 1] - adj_ptr[n]);
        for (int s = 0; s < K; s++) cnt[s] = 0;
        for (int64_t i = ib; i < ie; i++)
            for (int b = 0; b < 10; b++) cnt[slots[i * kSlotStride + b]]++;
        int pos = 0;
        for (int s = 0; s < K; s++) {
            const int c = cnt[s];
            cnt[s] = (uint16_t)pos;
            pos += c;
        }
        uint16_t *out = codes + 10 * ib;
        for (int64_t i = ib; i < ie; i++)
            for (int b = 0; b < 10; b++) {
                const int s = slots[i * kSlotStride + b];
                out[cnt[s]++] = (uint16_t)(b | ((int)(i - i0) << 4));
            }
        // after placement cnt[s] is the end of slot s, so slot s starts at cnt[s - 1]
        for (int s = 0; s < K; s++) out[s == 0 ? 0 : cnt[s - 1]] |= (uint16_t)kCodeSeg;
        out[0] |= (uint16_t)kCodeRow;
    }
}

int sm_count_seg() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

constexpr int kBI = 24, kBS = 128;     // structured meshes: a vertex row (24 incidences, 65 slots) per batch
constexpr int kBIw = 64, kBSw = 255;   // any mesh within the engine's per-node limits

}  // namespace

bool build_ns_seg_plan(NSSegPlan &P, const Graph &g, const int64_t *padj_ptr, const int32_t *padj,
                       const int32_t *vmap, cudaStream_t s) {
    P = NSSegPlan{};
    const int64_t nn = g.nrow_nodes;
    if (!vmap || nn <= 0 || g.max_inc > kBIw || g.max_adj > kBSw) return false;
    std::vector<int64_t> ip(nn + 1), ap(nn + 1);
    FEDD_CUDA(cudaMemcpyAsync(ip.data(), g.inc_ptr.p, (nn + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaMemcpyAsync(ap.data(), g.adj_ptr.p, (nn + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    const bool wide = g.max_inc > kBI || g.max_adj > kBS;
    const int BI = wide ? kBIw : kBI, BS = wide ? kBSw : kBS;
    // batches: consecutive row nodes with at most BI incidences, BS slots and 32 rows
    std::vector<int32_t> bn;
    bn.push_back(0);
    int cur_i = 0, cur_s = 0, cur_r = 0;
    for (int64_t n = 0; n < nn; n++) {
        const int m = (int)(ip[n + 1] - ip[n]), K = (int)(ap[n + 1] - ap[n]);
        if (cur_r > 0 && (cur_i + m > BI || cur_s + K > BS || cur_r == 32)) {
            bn.push_back((int32_t)n);
            cur_i = cur_s = cur_r = 0;
        }
        cur_i += m;
        cur_s += K;
        cur_r++;
    }
    bn.push_back((int32_t)nn);
    DBuf<int> bad;
    bad.alloc(1);
    bad.zero(s);
    P.pslot.alloc((size_t)std::max<int64_t>(g.n_adj, 1));
    k_seg_pslot<<<ceil_div(nn, 256), 256, 0, s>>>(nn, g.adj_ptr.p, g.adj.p, padj_ptr, padj, vmap, P.pslot.p, bad.p);
    FEDD_CUDA(cudaGetLastError());
    int hb = 0;
    FEDD_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof hb, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    if (hb) {
        P = NSSegPlan{};
        return false;
    }
    P.nbatch = (int64_t)bn.size() - 1;
    P.wide = wide;
    P.batch_node.upload(bn.data(), bn.size(), s);
    P.h_batch_node = bn;
    P.codes.alloc((size_t)std::max<int64_t>(10 * g.n_inc, 2));
    k_seg_codes<<<ceil_div(P.nbatch, 128), 128, 0, s>>>(P.batch_node.p, P.nbatch, g.inc_ptr.p, g.slots.p,
                                                         g.adj_ptr.p, P.codes.p);
    FEDD_CUDA(cudaGetLastError());
    FEDD_CUDA(cudaStreamSynchronize(s));
    P.ok = true;
    return true;
}

void launch_ns_seg_rows(const NSSegPlan &P, const Graph &g, const int64_t *padj_ptr, const int32_t *vmap,
                        const float *rec, const float *d_tables, const int64_t *rowptr00, const int64_t *rowptr01,
                        const int64_t *rowptr10, double *vals00, double *vals01, double *vals10, double *res_u,
                        double *res_p, float dens, int newton, int want_jac, int64_t b_begin, int64_t b_end,
                        unsigned long long *work, cudaStream_t s, LaunchCounter &lc) {
    if (b_end < 0) b_end = P.nbatch;
    if (b_end <= b_begin) return;
    SegArgs A{};
    A.batch_node = P.batch_node.p;
    A.codes = P.codes.p;
    A.pslot = P.pslot.p;
    A.inc_ptr = g.inc_ptr.p;
    A.inc = g.inc.p;
    A.adj_ptr = g.adj_ptr.p;
    A.padj_ptr = padj_ptr;
    A.vmap = vmap;
    A.rec = rec;
    A.gtab = d_tables;
    A.rowptr00 = rowptr00;
    A.rowptr01 = rowptr01;
    A.rowptr10 = rowptr10;
    A.vals00 = want_jac ? vals00 : nullptr;
    A.vals01 = vals01;
    A.vals10 = vals10;
    A.res_u = res_u;
    A.res_p = res_p;
    A.dens = dens;
    A.newton = newton;
    A.b_begin = b_begin;
    A.b_end = b_end;
    A.work = work;
    auto run = [&](auto kern, int per_warp) {
        const int warps = (int)std::max<size_t>(
            1, std::min<size_t>(12, (227 * 1024 - kTabFloats * sizeof(float)) / ((size_t)per_warp * sizeof(float))));
        const size_t smem = ((size_t)kTabFloats + (size_t)warps * per_warp) * sizeof(float);
        FEDD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        FEDD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * warps, smem));
        const unsigned grid = (unsigned)std::min<int64_t>((b_end - b_begin + warps - 1) / warps,
                                                          (int64_t)sm_count_seg() * std::max(per_sm, 1));
        FEDD_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned long long), s));
        kern<<<grid, 32 * warps, smem, s>>>(A);
        FEDD_CUDA(cudaGetLastError());
    };
    if (P.wide)
        run(k_ns_seg_rows<kBIw, kBSw>, SegCfg<kBIw, kBSw>::kPerWarp);
    else
        run(k_ns_seg_rows<kBI, kBS>, SegCfg<kBI, kBS>::kPerWarp);
    lc.n++;
}

}  // namespace fedd
