// k_mlp.cu -- training of the learned warm start on the GPU: sample
// statistics, initialisation, forward and backward passes over batches of
// recorded contacts, and Adam.
//
// Samples are recorded by the solver itself (features at assembly, converged
// impulses after the velocity solve). The loss is the mean squared error of
// the network's output against the normalised impulses, averaged over the
// batch and the three outputs. Weights are read in bf16 (the precision
// inference uses) and every sum accumulates in fp32; the fp32 master weights
// take the Adam updates. The hidden layer's three 64 x 64 x 64 products per
// tile (forward, weight gradient, back-propagated gradient) run on the tensor
// cores with bf16 operands; the other layers (24 inputs, 3 outputs) on the
// fp32 pipes.
#include <cstdint>
#include <cuda_runtime.h>

#include "mlp.cuh"

namespace npgpu_dev {

constexpr int kTile = 64;            // samples per block of the gradient kernel
constexpr int kMlpThreads = 256;

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    // A 32-bit integer hash (the finaliser of MurmurHash3).
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}

// Tensor-core tiles for the 64 x 64 x 64 products of the hidden layer:
// operands in shared memory as bf16 with a padded row of kLd elements, fp32
// accumulation (mma.sync m16n8k16; fragment layout of the PTX ISA:
// g = lane / 4, t = lane % 4; A rows g and g + 8, columns 2t, 2t + 1 (+ 8);
// B column g, rows 2t, 2t + 1 (+ 8); C rows g, g + 8, columns 2t, 2t + 1).
constexpr int kLd = 72;

// c += A[m0 .. m0 + 16][0 .. 64) * B[0 .. 64)[n0 .. n0 + 8), with A row-major
// and B given as Bt[n][k] (both bf16, leading dimension kLd).
__device__ __forceinline__ void mma_16x8x64(const __nv_bfloat16* A, const __nv_bfloat16* Bt, int m0, int n0, float* c) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int k0 = 0; k0 < 64; k0 += 16) {
        const uint32_t a0 = *reinterpret_cast<const uint32_t*>(A + (m0 + g) * kLd + k0 + 2 * t);
        const uint32_t a1 = *reinterpret_cast<const uint32_t*>(A + (m0 + g + 8) * kLd + k0 + 2 * t);
        const uint32_t a2 = *reinterpret_cast<const uint32_t*>(A + (m0 + g) * kLd + k0 + 8 + 2 * t);
        const uint32_t a3 = *reinterpret_cast<const uint32_t*>(A + (m0 + g + 8) * kLd + k0 + 8 + 2 * t);
        const uint32_t b0 = *reinterpret_cast<const uint32_t*>(Bt + (n0 + g) * kLd + k0 + 2 * t);
        const uint32_t b1 = *reinterpret_cast<const uint32_t*>(Bt + (n0 + g) * kLd + k0 + 8 + 2 * t);
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
            "{%0, %1, %2, %3};"
            : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
}

// One 64 x 64 product on the block's 8 warps: warp w owns rows 16 (w / 2) and
// columns 32 (w % 2) .. + 32, four 16 x 8 tiles. f(row, col, value) receives
// every output element once.
template <class F>
__device__ __forceinline__ void mma_64x64x64(const __nv_bfloat16* A, const __nv_bfloat16* Bt, F f) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int m0 = (warp >> 1) * 16;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int n0 = (warp & 1) * 32 + q * 8;
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        mma_16x8x64(A, Bt, m0, n0, c);
        f(m0 + g, n0 + 2 * t, c[0]);
        f(m0 + g, n0 + 2 * t + 1, c[1]);
        f(m0 + g + 8, n0 + 2 * t, c[2]);
        f(m0 + g + 8, n0 + 2 * t + 1, c[3]);
    }
}

// The inference copy of the parameters: weights rounded to bf16 (nearest,
// ties to even), biases and normalisation as they are.
__global__ void k_mlp_to_dev(const float* __restrict__ prm, MlpDev* net) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParams; i += gridDim.x * blockDim.x) {
        float v = prm[i];
        if (i < kMlpB1) net->w1[i - kMlpW1] = __float2bfloat16_rn(v);
        else if (i < kMlpW2) net->b1[i - kMlpB1] = v;
        else if (i < kMlpB2) net->w2[i - kMlpW2] = __float2bfloat16_rn(v);
        else if (i < kMlpW3) net->b2[i - kMlpB2] = v;
        else if (i < kMlpB3) net->w3[i - kMlpW3] = __float2bfloat16_rn(v);
        else if (i < kMlpTrainable) net->b3[i - kMlpB3] = v;
        else if (i < kMlpXInvStd) net->x_mean[i - kMlpXMean] = v;
        else if (i < kMlpYMean) net->x_inv_std[i - kMlpXInvStd] = v;
        else if (i < kMlpYStd) net->y_mean[i - kMlpYMean] = v;
        else net->y_std[i - kMlpYStd] = v;
    }
}

// Sums and sums of squares of the 27 sample columns (features, impulses).
__global__ void k_mlp_stats(const float* __restrict__ samples, uint32_t n, double* acc) {
    constexpr int C = kMlpIn + kMlpOut;
    double s[C], q[C];
    for (int c = 0; c < C; ++c) s[c] = q[c] = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* r = samples + (size_t)i * kMlpSampleFloats;
        for (int c = 0; c < C; ++c) {
            double v = r[c];
            s[c] += v;
            q[c] += v * v;
        }
    }
    for (int c = 0; c < C; ++c) {
        double a = s[c], b = q[c];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&acc[c], a);
            atomicAdd(&acc[C + c], b);
        }
    }
}

// Normalisation from the column statistics; a column without spread gets a
// zero scale (its feature is then constant 0 for the network).
__global__ void k_mlp_norm(const double* acc, uint32_t n, float* prm) {
    constexpr int C = kMlpIn + kMlpOut;
    int c = threadIdx.x;
    if (c >= C) return;
    double mean = acc[c] / (double)n;
    double var = acc[C + c] / (double)n - mean * mean;
    double sd = var > 0.0 ? sqrt(var) : 0.0;
    if (c < kMlpIn) {
        prm[kMlpXMean + c] = (float)mean;
        prm[kMlpXInvStd + c] = sd > 1e-12 ? (float)(1.0 / sd) : 0.0f;
    } else {
        prm[kMlpYMean + c - kMlpIn] = (float)mean;
        prm[kMlpYStd + c - kMlpIn] = sd > 1e-12 ? (float)sd : 1.0f;
    }
}

// He-uniform weights, zero biases.
__global__ void k_mlp_init(float* prm, uint32_t seed) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpTrainable; i += gridDim.x * blockDim.x) {
        int fan_in;
        bool bias = false;
        if (i < kMlpB1) fan_in = kMlpIn;
        else if (i < kMlpW2) bias = true, fan_in = 1;
        else if (i < kMlpB2) fan_in = kMlpHidden;
        else if (i < kMlpW3) bias = true, fan_in = 1;
        else if (i < kMlpB3) fan_in = kMlpHidden;
        else bias = true, fan_in = 1;
        float u = (float)(mix32(seed * 0x9e3779b9u + (uint32_t)i) >> 8) * (1.0f / 16777216.0f);   // [0, 1)
        float a = sqrtf(6.0f / (float)fan_in);
        prm[i] = bias ? 0.0f : (2.0f * u - 1.0f) * a;
    }
}

// Gradient of the batch loss with respect to every trainable parameter,
// accumulated into grad (zeroed by the caller), and the loss into *loss.
// Block b takes samples [b * 64, b * 64 + 64) of the batch; batch sample i is
// recorded sample idx(i) = hash(seed, step, i) mod n, or i itself when
// seed == 0 (a fixed batch, for gradient checks).
__global__ void __launch_bounds__(kMlpThreads) k_mlp_grad(const MlpDev* __restrict__ net,
                                                          const float* __restrict__ samples, uint32_t n,
                                                          uint32_t batch, uint32_t seed, uint32_t step, float* grad,
                                                          double* loss) {
    extern __shared__ float sm[];
    float* W1T = sm;                                   // [24][64]
    float* W3 = W1T + kMlpIn * kMlpHidden;             // [3][64]
    float* B1 = W3 + kMlpOut * kMlpHidden;
    float* B2 = B1 + kMlpHidden;
    float* B3 = B2 + kMlpHidden;                       // 4 floats
    float* X = B3 + 4;                                 // [64][24]
    float* T = X + kTile * kMlpIn;                     // [64][3] normalised targets
    float* H1 = T + kTile * 4;                         // [64][64]
    float* H2 = H1 + kTile * kMlpHidden;               // [64][64], later dH1
    float* D2 = H2 + kTile * kMlpHidden;               // [64][64] dH2
    float* DY = D2 + kTile * kMlpHidden;               // [64][3]
    // bf16 operands of the hidden layer's products (rows padded to kLd).
    __nv_bfloat16* H1b = reinterpret_cast<__nv_bfloat16*>(DY + kTile * 4);   // H1[s][i]
    __nv_bfloat16* H1Tb = H1b + kTile * kLd;                                   // H1[s][i] at [i][s]
    __nv_bfloat16* W2b = H1Tb + kTile * kLd;                                   // W2[j][i]
    __nv_bfloat16* W2Tb = W2b + kTile * kLd;                                   // W2[j][i] at [i][j]
    __nv_bfloat16* D2b = W2Tb + kTile * kLd;                                   // dH2[s][j]
    __nv_bfloat16* D2Tb = D2b + kTile * kLd;                                   // dH2[s][j] at [j][s]
    __shared__ double s_loss[kMlpThreads / 32];
    const int tid = threadIdx.x;

    for (int i = tid; i < kMlpHidden * kMlpIn; i += kMlpThreads) {
        int j = i / kMlpIn, k = i % kMlpIn;
        W1T[k * kMlpHidden + j] = bf(net->w1, i);
    }
    for (int i = tid; i < kMlpHidden * kMlpHidden; i += kMlpThreads) {
        int j = i / kMlpHidden, k = i % kMlpHidden;
        W2b[j * kLd + k] = net->w2[i];
        W2Tb[k * kLd + j] = net->w2[i];
    }
    for (int i = tid; i < kMlpOut * kMlpHidden; i += kMlpThreads) W3[i] = bf(net->w3, i);
    for (int i = tid; i < kMlpHidden; i += kMlpThreads) {
        B1[i] = net->b1[i];
        B2[i] = net->b2[i];
    }
    if (tid < kMlpOut) B3[tid] = net->b3[tid];

    const uint32_t first = blockIdx.x * kTile;
    const int rows = (int)min((uint32_t)kTile, batch - first);
    for (int e = tid; e < kTile * kMlpIn; e += kMlpThreads) {
        int s = e / kMlpIn, i = e % kMlpIn;
        float v = 0.0f;
        if (s < rows) {
            uint32_t bi = first + s;
            uint32_t idx = seed == 0u ? bi : mix32(seed ^ mix32(step * 0x9e3779b9u + bi)) % n;
            v = (samples[(size_t)idx * kMlpSampleFloats + i] - net->x_mean[i]) * net->x_inv_std[i];
        }
        X[e] = v;
    }
    for (int e = tid; e < kTile * kMlpOut; e += kMlpThreads) {
        int s = e / kMlpOut, o = e % kMlpOut;
        float v = 0.0f;
        if (s < rows) {
            uint32_t bi = first + s;
            uint32_t idx = seed == 0u ? bi : mix32(seed ^ mix32(step * 0x9e3779b9u + bi)) % n;
            v = (samples[(size_t)idx * kMlpSampleFloats + kMlpIn + o] - net->y_mean[o]) / net->y_std[o];
        }
        T[s * 4 + o] = v;
    }
    __syncthreads();

    // Forward.
    for (int e = tid; e < kTile * kMlpHidden; e += kMlpThreads) {
        int s = e / kMlpHidden, j = e % kMlpHidden;
        float a = B1[j];
        for (int i = 0; i < kMlpIn; ++i) a = a + W1T[i * kMlpHidden + j] * X[s * kMlpIn + i];
        const float h = a > 0.0f ? a : 0.0f;
        H1[e] = h;
        const __nv_bfloat16 hb = __float2bfloat16_rn(h);
        H1b[s * kLd + j] = hb;
        H1Tb[j * kLd + s] = hb;
    }
    __syncthreads();
    // Hidden layer 2 on the tensor cores: H2 = relu(H1 W2^T + b2).
    mma_64x64x64(H1b, W2b, [&](int s, int j, float v) {
        const float a = v + B2[j];
        H2[s * kMlpHidden + j] = a > 0.0f ? a : 0.0f;
    });
    __syncthreads();
    double lsum = 0.0;
    const float scale = 2.0f / (float)(batch * kMlpOut);
    for (int e = tid; e < kTile * kMlpOut; e += kMlpThreads) {
        int s = e / kMlpOut, o = e % kMlpOut;
        float d = 0.0f;
        if (s < rows) {
            float y = B3[o];
            for (int j = 0; j < kMlpHidden; ++j) y = y + W3[o * kMlpHidden + j] * H2[s * kMlpHidden + j];
            float r = y - T[s * 4 + o];
            lsum += (double)r * (double)r;
            d = r * scale;
        }
        DY[s * 4 + o] = d;
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0) s_loss[tid >> 5] = lsum;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int k = 0; k < kMlpThreads / 32; ++k) t += s_loss[k];
        atomicAdd(loss, t / (double)(batch * kMlpOut));
    }

    // Backward: output layer.
    for (int e = tid; e < kMlpOut * kMlpHidden + kMlpOut; e += kMlpThreads) {
        float g = 0.0f;
        if (e < kMlpOut * kMlpHidden) {
            int o = e / kMlpHidden, j = e % kMlpHidden;
            for (int s = 0; s < kTile; ++s) g = g + DY[s * 4 + o] * H2[s * kMlpHidden + j];
            atomicAdd(&grad[kMlpW3 + e], g);
        } else {
            int o = e - kMlpOut * kMlpHidden;
            for (int s = 0; s < kTile; ++s) g = g + DY[s * 4 + o];
            atomicAdd(&grad[kMlpB3 + o], g);
        }
    }
    for (int e = tid; e < kTile * kMlpHidden; e += kMlpThreads) {
        int s = e / kMlpHidden, j = e % kMlpHidden;
        float g = 0.0f;
        for (int o = 0; o < kMlpOut; ++o) g = g + DY[s * 4 + o] * W3[o * kMlpHidden + j];
        const float d = H2[e] > 0.0f ? g : 0.0f;
        D2[e] = d;
        const __nv_bfloat16 db = __float2bfloat16_rn(d);
        D2b[s * kLd + j] = db;
        D2Tb[j * kLd + s] = db;
    }
    __syncthreads();
    // Hidden layer 2 backward on the tensor cores: dW2[j][i] = sum_s
    // dH2[s][j] H1[s][i]; dH1 = (dH2 W2) masked by H1 > 0, into H2's space.
    float* D1 = H2;
    mma_64x64x64(D2Tb, H1Tb, [&](int j, int i, float v) { atomicAdd(&grad[kMlpW2 + j * kMlpHidden + i], v); });
    for (int j = tid; j < kMlpHidden; j += kMlpThreads) {
        float g = 0.0f;
        for (int s = 0; s < kTile; ++s) g = g + D2[s * kMlpHidden + j];
        atomicAdd(&grad[kMlpB2 + j], g);
    }
    mma_64x64x64(D2b, W2Tb, [&](int s, int i, float v) {
        D1[s * kMlpHidden + i] = H1[s * kMlpHidden + i] > 0.0f ? v : 0.0f;
    });
    __syncthreads();
    // Hidden layer 1.
    for (int e = tid; e < kMlpHidden * kMlpIn; e += kMlpThreads) {
        int j = e / kMlpIn, i = e % kMlpIn;
        float g = 0.0f;
        for (int s = 0; s < kTile; ++s) g = g + D1[s * kMlpHidden + j] * X[s * kMlpIn + i];
        atomicAdd(&grad[kMlpW1 + e], g);
    }
    for (int j = tid; j < kMlpHidden; j += kMlpThreads) {
        float g = 0.0f;
        for (int s = 0; s < kTile; ++s) g = g + D1[s * kMlpHidden + j];
        atomicAdd(&grad[kMlpB1 + j], g);
    }
}

constexpr size_t kGradSmem = sizeof(float) * (kMlpIn * kMlpHidden + kMlpOut * kMlpHidden +
                                              2 * kMlpHidden + 4 + kTile * kMlpIn + kTile * 4 +
                                              3 * kTile * kMlpHidden + kTile * 4) +
                             sizeof(__nv_bfloat16) * 6 * kTile * kLd;

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on the fp32 master weights, then
// the inference copy.
__global__ void k_mlp_adam(float* prm, float* m1, float* m2, const float* grad, float lr, uint32_t t, MlpDev* net) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpTrainable; i += gridDim.x * blockDim.x) {
        float g = grad[i];
        float a = b1 * m1[i] + (1.0f - b1) * g;
        float b = b2 * m2[i] + (1.0f - b2) * g * g;
        m1[i] = a;
        m2[i] = b;
        float v = prm[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        prm[i] = v;
        if (i < kMlpB1) net->w1[i - kMlpW1] = __float2bfloat16_rn(v);
        else if (i < kMlpW2) net->b1[i - kMlpB1] = v;
        else if (i < kMlpB2) net->w2[i - kMlpW2] = __float2bfloat16_rn(v);
        else if (i < kMlpW3) net->b2[i - kMlpB2] = v;
        else if (i < kMlpB3) net->w3[i - kMlpW3] = __float2bfloat16_rn(v);
        else net->b3[i - kMlpB3] = v;
    }
}

// ---- launchers ----
cudaError_t mlp_upload(const float* prm_dev, MlpDev* net, cudaStream_t st) {
    k_mlp_to_dev<<<(kMlpParams + 255) / 256, 256, 0, st>>>(prm_dev, net);
    return cudaGetLastError();
}

cudaError_t mlp_normalise(const float* samples, uint32_t n, double* acc, float* prm, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double) * 2 * (kMlpIn + kMlpOut), st);
    if (e != cudaSuccess) return e;
    unsigned blocks = (n + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    if (blocks < 1) blocks = 1;
    k_mlp_stats<<<blocks, 256, 0, st>>>(samples, n, acc);
    k_mlp_norm<<<1, 32, 0, st>>>(acc, n, prm);
    return cudaGetLastError();
}

cudaError_t mlp_init(float* prm, uint32_t seed, cudaStream_t st) {
    k_mlp_init<<<(kMlpTrainable + 255) / 256, 256, 0, st>>>(prm, seed);
    return cudaGetLastError();
}

cudaError_t mlp_grad(const MlpDev* net, const float* samples, uint32_t n, uint32_t batch, uint32_t seed, uint32_t step,
                     float* grad, double* loss, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(grad, 0, sizeof(float) * kMlpTrainable, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(loss, 0, sizeof(double), st);
    if (e != cudaSuccess) return e;
    k_mlp_grad<<<(batch + kTile - 1) / kTile, kMlpThreads, kGradSmem, st>>>(net, samples, n, batch, seed, step, grad,
                                                                            loss);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float* prm, float* m1, float* m2, const float* grad, float lr, uint32_t t, MlpDev* net,
                     cudaStream_t st) {
    k_mlp_adam<<<(kMlpTrainable + 255) / 256, 256, 0, st>>>(prm, m1, m2, grad, lr, t, net);
    return cudaGetLastError();
}

}  // namespace npgpu_dev
