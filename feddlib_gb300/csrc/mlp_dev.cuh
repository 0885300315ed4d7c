// mlp_dev.cuh -- scalar (one thread per point) evaluation of the strain-energy
// surrogate with first and second input derivatives.  Used by the law
// evaluation entry point that scores the surrogate against the law; the quadrature-point hot
// path uses the tensor-core kernel in mlp.cu.
#pragma once
#include <cuda_bf16.h>

#include "kernels.cuh"

namespace fedd {

__device__ __forceinline__ float softplus_f(float z) { return z > 20.0f ? z : log1pf(__expf(z)); }
__device__ __forceinline__ float sigmoid_f(float z) { return 1.0f / (1.0f + __expf(-z)); }

// input k of the network: (a - in_shift_k) in_scale_k, or for the inputs
// flagged in in_clamp max(a - in_shift_k, 0)^2 in_scale_k; dk = dx_k / da and
// d2k = d2x_k / da2 (all zero on the clamped side, where the surrogate and
// its derivatives vanish; dk -> 0 at the shift, so the stress stays
// continuous there)
__device__ __forceinline__ float mlp_input(const MLPDev &m, int k, float a, float &dk, float &d2k) {
    const float e = a - m.in_shift[k];
    if ((m.in_clamp >> k) & 1) {
        if (!(e > 0.0f)) {
            dk = d2k = 0.0f;
            return 0.0f;
        }
        dk = 2.0f * e * m.in_scale[k];
        d2k = 2.0f * m.in_scale[k];
        return e * e * m.in_scale[k];
    }
    dk = m.in_scale[k];
    d2k = 0.0f;
    return e * m.in_scale[k];
}

// net(x) = w3 . sp(W2 sp(W1 x + b1) + b2) + b3 and its gradient g and
// Hessian h (4x4, row-major) with respect to x.
__device__ __forceinline__ void mlp_eval_scalar(const MLPDev &m, const float *x, float &y, float *g, float *h) {
    const __nv_bfloat16 *W1 = (const __nv_bfloat16 *)m.W1, *W2 = (const __nv_bfloat16 *)m.W2,
                        *w3 = (const __nv_bfloat16 *)m.w3;
    const int H = m.hidden;
    float yy = m.b3, gg[4] = {0, 0, 0, 0}, hh[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < H; j++) {
        float z = m.b2[j], dz[4] = {0, 0, 0, 0}, d2z[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < H; i++) {
            float wi[4];
            float z1 = m.b1[i];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                wi[k] = __bfloat162float(W1[4 * i + k]);
                z1 = fmaf(wi[k], x[k], z1);
            }
            float s1 = sigmoid_f(z1), t1 = s1 * (1.0f - s1), h1 = softplus_f(z1);
            float wji = __bfloat162float(W2[H * j + i]);
            z = fmaf(wji, h1, z);
            int kl = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                dz[k] = fmaf(wji, s1 * wi[k], dz[k]);
#pragma unroll
                for (int l = k; l < 4; l++, kl++) d2z[kl] = fmaf(wji, t1 * wi[k] * wi[l], d2z[kl]);
            }
        }
        float s2 = sigmoid_f(z), t2 = s2 * (1.0f - s2), c = __bfloat162float(w3[j]);
        yy = fmaf(c, softplus_f(z), yy);
        int kl = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            gg[k] = fmaf(c * s2, dz[k], gg[k]);
#pragma unroll
            for (int l = k; l < 4; l++, kl++) hh[kl] = fmaf(c, t2 * dz[k] * dz[l] + s2 * d2z[kl], hh[kl]);
        }
    }
    y = yy;
    int kl = 0;
    for (int k = 0; k < 4; k++) {
        g[k] = gg[k];
        for (int l = k; l < 4; l++, kl++) {
            h[4 * k + l] = hh[kl];
            h[4 * l + k] = hh[kl];
        }
    }
}

}  // namespace fedd
