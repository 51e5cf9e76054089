// mlp.cuh -- the learned warm start: contact features, the network and its
// forward pass as constraint assembly runs it.
//
// A contact with no impulse-cache entry (a new contact) gets its starting
// impulses (normal, tangent 1, tangent 2) from a 24 -> 64 -> 64 -> 3
// perceptron with ReLU hidden layers, bf16 weights and fp32 accumulation. The
// prediction is checked in the warm-start sweep of the velocity solver: a
// contact whose predicted start leaves a larger local residual than the zero
// start falls back to the zero start, so the SOR-Prox iterations decide the result.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

#include "world_dev.cuh"

namespace npgpu_dev {

constexpr int kMlpIn = 24;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 3;
// Parameters in their fp32 layout (npgpu_mlp_set / npgpu_mlp_get):
//   W1[64][24] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]
//   x_mean[24] x_inv_std[24] y_mean[3] y_std[3]
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHidden * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpOut * kMlpHidden;
constexpr int kMlpTrainable = kMlpB3 + kMlpOut;               // 5955
constexpr int kMlpXMean = kMlpTrainable;
constexpr int kMlpXInvStd = kMlpXMean + kMlpIn;
constexpr int kMlpYMean = kMlpXInvStd + kMlpIn;
constexpr int kMlpYStd = kMlpYMean + kMlpOut;
constexpr int kMlpParams = kMlpYStd + kMlpOut;                // 6009
constexpr int kMlpSampleFloats = kMlpIn + kMlpOut + 1;        // features, converged impulses, new-contact flag

// The network as inference reads it: weights rounded to bf16, biases and
// normalisation in fp32.
struct MlpDev {
    __nv_bfloat16 w1[kMlpHidden * kMlpIn];
    __nv_bfloat16 w2[kMlpHidden * kMlpHidden];
    __nv_bfloat16 w3[kMlpOut * kMlpHidden];
    float b1[kMlpHidden], b2[kMlpHidden], b3[kMlpOut];
    float x_mean[kMlpIn], x_inv_std[kMlpIn], y_mean[kMlpOut], y_std[kMlpOut];
};

__device__ __forceinline__ float bf(const __nv_bfloat16* p, int i) { return __bfloat162float(p[i]); }

// Forward pass of one contact: every sum runs in index order in fp32, without
// fused multiply-add (the oracle evaluates the same sequence).
__device__ __forceinline__ void mlp_forward(const MlpDev* __restrict__ net, const float* feat, float* lam_out) {
    float x[kMlpIn];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) x[i] = (feat[i] - net->x_mean[i]) * net->x_inv_std[i];
    float h1[kMlpHidden];
#pragma unroll 4
    for (int j = 0; j < kMlpHidden; ++j) {
        float a = net->b1[j];
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i) a = a + bf(net->w1, j * kMlpIn + i) * x[i];
        h1[j] = a > 0.0f ? a : 0.0f;
    }
    float y[kMlpOut];
#pragma unroll
    for (int o = 0; o < kMlpOut; ++o) y[o] = net->b3[o];
#pragma unroll 1
    for (int j = 0; j < kMlpHidden; ++j) {
        float a = net->b2[j];
#pragma unroll
        for (int i = 0; i < kMlpHidden; ++i) a = a + bf(net->w2, j * kMlpHidden + i) * h1[i];
        float h = a > 0.0f ? a : 0.0f;
#pragma unroll
        for (int o = 0; o < kMlpOut; ++o) y[o] = y[o] + bf(net->w3, o * kMlpHidden + j) * h;
    }
#pragma unroll
    for (int o = 0; o < kMlpOut; ++o) lam_out[o] = y[o] * net->y_std[o] + net->y_mean[o];
}

// The 24 features of one contact, from its three assembled rows (RF_* layout):
//   0-2   rhs of the normal, tangent 1, tangent 2 rows (after restitution and
//         the speculative term)
//   3-5   r of the three rows (inverse effective masses' reciprocals)
//   6     depth + both margins
//   7, 8  inverse masses of body 1 and 2 (0 without dofs)
//   9-11  angular terms J1.ang . WJ1.ang of the three rows, body 1
//   12-14 the same for body 2
//   15    friction coefficient
//   16    gravity . n * dt
//   17    contacts in the manifold
//   18,19 solver manifolds of body 1 and 2 (0 without dofs)
//   20    max(0, -r_n rhs_n): the normal impulse of the contact alone
//   21,22 -r_t rhs_t of the tangent rows
//   23    r_n (gravity . n * dt)
__device__ __forceinline__ void mlp_features(const float* rn, const float* rt1, const float* rt2, float depth,
                                             float im1, float im2, float mu, float gn_dt, float nc, float k1, float k2,
                                             float* f) {
    const float* rows[3] = {rn, rt1, rt2};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        f[r] = rows[r][RF_RHS];
        f[3 + r] = rows[r][RF_R];
    }
    f[6] = depth;
    f[7] = im1;
    f[8] = im2;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float a1 = 0.0f, a2 = 0.0f;
#pragma unroll
        for (int k = 3; k < 6; ++k) {
            a1 = a1 + rows[r][RF_J1 + k] * rows[r][RF_WJ1 + k];
            a2 = a2 + rows[r][RF_J2 + k] * rows[r][RF_WJ2 + k];
        }
        f[9 + r] = a1;
        f[12 + r] = a2;
    }
    f[15] = mu;
    f[16] = gn_dt;
    f[17] = nc;
    f[18] = k1;
    f[19] = k2;
    float iso = -(f[3] * f[0]);
    f[20] = iso > 0.0f ? iso : 0.0f;
    f[21] = -(f[4] * f[1]);
    f[22] = -(f[5] * f[2]);
    f[23] = f[3] * gn_dt;
}

// Starting impulses of a new contact from the network's output: the normal
// impulse is kept non-negative and the friction impulses inside the pyramid
// of the normal one.
__device__ __forceinline__ void mlp_project(float mu, float* lam) {
    float ln = lam[0] > 0.0f ? lam[0] : 0.0f;
    float mx = mu * ln;
    lam[0] = ln;
#pragma unroll
    for (int s = 1; s < 3; ++s) lam[s] = lam[s] < -mx ? -mx : (lam[s] > mx ? mx : lam[s]);
}

}  // namespace npgpu_dev
