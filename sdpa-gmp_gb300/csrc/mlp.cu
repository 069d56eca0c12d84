// CUDA kernels of the learned parameter proposal (forward pass, backward pass with
// gradient accumulation, Adam) and its C ABI.  One CTA of 64 threads takes a tile of
// 32 samples: thread j owns hidden unit j, the weights sit in shared memory with the
// 64 x 64 matrices at a padded row stride of 65 so that both the forward (unit-major)
// and the backward (input-major) sweeps read them without bank conflicts, and the
// activations of the tile are kept for the backward sweep, which overwrites them in
// place with the layer deltas.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <random>
#include <vector>

#include "capi_util.cuh"
#include "mlp.cuh"
#include "sdpg.h"

static_assert(SDPG_POLICY_INPUTS == sdpg::kPolIn, "header and kernels disagree on the input width");
static_assert(SDPG_POLICY_OUTPUTS == sdpg::kPolOut, "header and kernels disagree on the output width");
static_assert(SDPG_POLICY_PARAMS == sdpg::kPolParams, "header and kernels disagree on the parameter count");
static_assert(SDPG_POLICY_SCALE == sdpg::kPolScale, "header and kernels disagree on the scaling block");

namespace sdpg {

namespace {

constexpr int kTile = 32;        // samples per CTA
constexpr int kThreads = kPolH;  // one thread per hidden unit
constexpr int kLd = kPolH + 1;   // padded row stride of the 64 x 64 weights

// shared-memory layout, in floats
constexpr int sW1 = 0;  // [64][kPolIn], read once into registers
constexpr int sB1 = sW1 + kPolH * kPolIn;
constexpr int sW2 = sB1 + kPolH;  // [64][65]
constexpr int sB2 = sW2 + kPolH * kLd;
constexpr int sW3 = sB2 + kPolH;  // [64][65]
constexpr int sB3 = sW3 + kPolH * kLd;
constexpr int sW4 = sB3 + kPolH;  // [2][64]
constexpr int sB4 = sW4 + kPolOut * kPolH;
constexpr int sSc = sB4 + kPolOut;          // scaling block
constexpr int sA0 = sSc + kPolScale;        // [32][kPolIn] standardised inputs
constexpr int sA1 = sA0 + kTile * kPolIn;   // [32][64] activations (then deltas)
constexpr int sA2 = sA1 + kTile * kPolH;
constexpr int sA3 = sA2 + kTile * kPolH;
constexpr int sY = sA3 + kTile * kPolH;     // [32][2] standardised outputs, then their gradients
constexpr int kSmemFloats = sY + kTile * kPolOut;
constexpr size_t kSmemBytes = kSmemFloats * sizeof(float);

// a_out[s][t] = tanh(b + sum_i W[t][i] a_in[s][i]) for the tile; W at row stride kLd
__device__ __forceinline__ void dense_tanh(const float *W, float b, const float *a_in, float *a_out, int t) {
    float w[kPolH];
#pragma unroll
    for (int i = 0; i < kPolH; ++i) w[i] = W[t * kLd + i];
    for (int s = 0; s < kTile; ++s) {
        float z = b;
#pragma unroll
        for (int i = 0; i < kPolH; ++i) z = fmaf(w[i], a_in[s * kPolH + i], z);
        a_out[s * kPolH + t] = tanhf(z);
    }
}

// Backward through one 64 -> 64 tanh layer.  d_out holds the deltas of the layer's
// output (dL/dz), a_in its input activations.  Accumulates dL/dW and dL/db into gW, gb
// and overwrites a_in with the deltas of the previous layer's pre-activations.
__device__ __forceinline__ void backward_dense(const float *W, float *a_in, const float *d_out, float *gW,
                                               float *gb, int t) {
    {
        float dj[kTile];
        float sb = 0.f;
#pragma unroll
        for (int s = 0; s < kTile; ++s) {
            dj[s] = d_out[s * kPolH + t];
            sb += dj[s];
        }
        atomicAdd(gb + t, sb);
        for (int i = 0; i < kPolH; ++i) {
            float g = 0.f;
#pragma unroll
            for (int s = 0; s < kTile; ++s) g = fmaf(dj[s], a_in[s * kPolH + i], g);
            atomicAdd(gW + t * kPolH + i, g);
        }
    }
    __syncthreads();  // every thread has read the input activations
    float wc[kPolH];
#pragma unroll
    for (int j = 0; j < kPolH; ++j) wc[j] = W[j * kLd + t];
    for (int s = 0; s < kTile; ++s) {
        float z = 0.f;
#pragma unroll
        for (int j = 0; j < kPolH; ++j) z = fmaf(wc[j], d_out[s * kPolH + j], z);
        const float a = a_in[s * kPolH + t];
        a_in[s * kPolH + t] = z * (1.f - a * a);
    }
    __syncthreads();
}

// Forward pass for a tile; with G set also the loss
//   sum over samples and outputs of mask * (y_std - t_std)^2 * inv_batch
// (standardised units) and its gradient, accumulated into G and *loss.
// Sample s of the tile is row perm[first + tile + s] of X/T/M (row first + tile + s
// without perm); Y, if set, receives the de-standardised outputs at index tile + s.
__global__ void __launch_bounds__(kThreads) policy_kernel(const float *__restrict__ P, const float *__restrict__ Sc,
                                                          const float *__restrict__ X, const float *__restrict__ T,
                                                          const float *__restrict__ M, const int *__restrict__ perm,
                                                          int first, int count, float inv_batch, float *__restrict__ Y,
                                                          float *__restrict__ G, float *__restrict__ loss) {
    extern __shared__ float sm[];
    const int t = threadIdx.x;
    for (int q = t; q < kPolH * kPolIn; q += kThreads) sm[sW1 + q] = P[kPolW1 + q];
    for (int q = t; q < kPolH * kPolH; q += kThreads) {
        const int j = q / kPolH, i = q % kPolH;
        sm[sW2 + j * kLd + i] = P[kPolW2 + q];
        sm[sW3 + j * kLd + i] = P[kPolW3 + q];
    }
    for (int q = t; q < kPolOut * kPolH; q += kThreads) sm[sW4 + q] = P[kPolW4 + q];
    sm[sB1 + t] = P[kPolB1 + t];
    sm[sB2 + t] = P[kPolB2 + t];
    sm[sB3 + t] = P[kPolB3 + t];
    if (t < kPolOut) sm[sB4 + t] = P[kPolB4 + t];
    if (t < kPolScale) sm[sSc + t] = Sc[t];
    __syncthreads();

    const int base = blockIdx.x * kTile;
    for (int q = t; q < kTile * kPolIn; q += kThreads) {
        const int s = q / kPolIn, i = q % kPolIn;
        const int idx = base + s;
        float v = 0.f;
        if (idx < count) {
            const int r = perm ? perm[first + idx] : first + idx;
            v = (X[(size_t)r * kPolIn + i] - sm[sSc + i]) / sm[sSc + kPolIn + i];
        }
        sm[sA0 + q] = v;
    }
    __syncthreads();
    {
        float w[kPolIn];
#pragma unroll
        for (int i = 0; i < kPolIn; ++i) w[i] = sm[sW1 + t * kPolIn + i];
        const float b = sm[sB1 + t];
        for (int s = 0; s < kTile; ++s) {
            float z = b;
#pragma unroll
            for (int i = 0; i < kPolIn; ++i) z = fmaf(w[i], sm[sA0 + s * kPolIn + i], z);
            sm[sA1 + s * kPolH + t] = tanhf(z);
        }
    }
    __syncthreads();
    dense_tanh(sm + sW2, sm[sB2 + t], sm + sA1, sm + sA2, t);
    __syncthreads();
    dense_tanh(sm + sW3, sm[sB3 + t], sm + sA2, sm + sA3, t);
    __syncthreads();

    // output layer: thread t = (sample t / 2, output t % 2)
    const int s = t >> 1, o = t & 1;
    const int idx = base + s;
    float yn = sm[sB4 + o];
#pragma unroll 8
    for (int i = 0; i < kPolH; ++i) yn = fmaf(sm[sW4 + o * kPolH + i], sm[sA3 + s * kPolH + i], yn);
    const float ym = sm[sSc + 2 * kPolIn + o], ys = sm[sSc + 2 * kPolIn + kPolOut + o];
    if (Y && idx < count) Y[(size_t)idx * kPolOut + o] = ym + ys * yn;
    if (!G) return;

    float d = 0.f, l = 0.f;
    if (idx < count) {
        const int r = perm ? perm[first + idx] : first + idx;
        const float mk = M[(size_t)r * kPolOut + o];
        const float e = yn - (T[(size_t)r * kPolOut + o] - ym) / ys;
        d = 2.f * mk * e * inv_batch;
        l = mk * e * e * inv_batch;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((t & 31) == 0) atomicAdd(loss, l);
    sm[sY + t] = d;
    __syncthreads();

    // output layer weights; then the deltas of the third hidden layer in place of a3
    {
        float g0 = 0.f, g1 = 0.f;
        for (int q = 0; q < kTile; ++q) {
            const float a = sm[sA3 + q * kPolH + t];
            g0 = fmaf(sm[sY + 2 * q], a, g0);
            g1 = fmaf(sm[sY + 2 * q + 1], a, g1);
        }
        atomicAdd(G + kPolW4 + t, g0);
        atomicAdd(G + kPolW4 + kPolH + t, g1);
        if (t < kPolOut) {
            float gb = 0.f;
            for (int q = 0; q < kTile; ++q) gb += sm[sY + 2 * q + t];
            atomicAdd(G + kPolB4 + t, gb);
        }
        const float w0 = sm[sW4 + t], w1 = sm[sW4 + kPolH + t];
        for (int q = 0; q < kTile; ++q) {
            const float a = sm[sA3 + q * kPolH + t];
            sm[sA3 + q * kPolH + t] = (w0 * sm[sY + 2 * q] + w1 * sm[sY + 2 * q + 1]) * (1.f - a * a);
        }
    }
    __syncthreads();
    backward_dense(sm + sW3, sm + sA2, sm + sA3, G + kPolW3, G + kPolB3, t);  // a2 <- delta2
    backward_dense(sm + sW2, sm + sA1, sm + sA2, G + kPolW2, G + kPolB2, t);  // a1 <- delta1
    {
        float g[kPolIn];
        float sb = 0.f;
#pragma unroll
        for (int i = 0; i < kPolIn; ++i) g[i] = 0.f;
        for (int q = 0; q < kTile; ++q) {
            const float dq = sm[sA1 + q * kPolH + t];
            sb += dq;
#pragma unroll
            for (int i = 0; i < kPolIn; ++i) g[i] = fmaf(dq, sm[sA0 + q * kPolIn + i], g[i]);
        }
        atomicAdd(G + kPolB1 + t, sb);
#pragma unroll
        for (int i = 0; i < kPolIn; ++i) atomicAdd(G + kPolW1 + t * kPolIn + i, g[i]);
    }
}

// Adam (Kingma & Ba 2015) on every parameter; clears the gradient for the next step.
__global__ void policy_adam_kernel(float *__restrict__ P, float *__restrict__ G, float *__restrict__ m1,
                                   float *__restrict__ m2, int n, float lr, float b1, float b2, float eps, float bc1,
                                   float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float v = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = v;
    P[i] -= lr * (a / bc1) / (sqrtf(v / bc2) + eps);
    G[i] = 0.f;
}

void ensure_smem(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    if (device < 0 || device >= 64) throw sdpg_error(SDPG_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (done[device]) return;
    SDPG_CUDA(cudaFuncSetAttribute(policy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes));
    done[device] = true;
}

void launch(const Policy &p, const float *X, const float *T, const float *M, const int *perm, int first, int count,
            float inv_batch, float *Y, float *G, float *loss, cudaStream_t s) {
    ensure_smem(p.device);
    SDPG_KT_BEGIN(s);
    policy_kernel<<<(count + kTile - 1) / kTile, kThreads, kSmemBytes, s>>>(p.params, p.scale, X, T, M, perm, first,
                                                                         count, inv_batch, Y, G, loss);
    SDPG_CHECK_LAUNCH_KT("policy_kernel", s);
}

Policy &get(sdpg_policy *h) {
    if (!h || !h->p.params) throw sdpg_error(SDPG_ERR_ARG, "null policy handle");
    SDPG_CUDA(cudaSetDevice(h->p.device));
    return h->p;
}

// Glorot-uniform weights from a fixed seed, zero biases, identity scaling.
void init_params(std::vector<float> &w, std::vector<float> &sc) {
    w.assign(kPolParams, 0.f);
    std::mt19937_64 g(12345);
    auto fill = [&](int off, int rows, int cols) {
        const double a = sqrt(6.0 / (rows + cols));
        std::uniform_real_distribution<double> u(-a, a);
        for (int q = 0; q < rows * cols; ++q) w[off + q] = (float)u(g);
    };
    fill(kPolW1, kPolH, kPolIn);
    fill(kPolW2, kPolH, kPolH);
    fill(kPolW3, kPolH, kPolH);
    fill(kPolW4, kPolOut, kPolH);
    sc.assign(kPolScale, 0.f);
    for (int i = 0; i < kPolIn; ++i) sc[kPolIn + i] = 1.f;
    for (int o = 0; o < kPolOut; ++o) sc[2 * kPolIn + kPolOut + o] = 1.f;
}

void check_scale(const float *sc) {
    for (int i = 0; i < kPolIn + kPolOut; ++i) {
        const float sd = i < kPolIn ? sc[kPolIn + i] : sc[2 * kPolIn + kPolOut + (i - kPolIn)];
        if (!(sd > 0.f) || !std::isfinite(sd)) throw sdpg_error(SDPG_ERR_ARG, "policy scales must be positive");
    }
}

struct DevFloats {
    float *p = nullptr;
    explicit DevFloats(size_t n) { SDPG_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(float))); }
    ~DevFloats() { cudaFree(p); }
};

}  // namespace

void policy_forward_device(const Policy &p, const float *x, int count, float *y, cudaStream_t s) {
    if (count <= 0) return;
    launch(p, x, nullptr, nullptr, nullptr, 0, count, 0.f, y, nullptr, nullptr, s);
}

}  // namespace sdpg

using namespace sdpg;

extern "C" {

int sdpg_policy_create(int device, sdpg_policy **out) {
    return sdpg_guard([&] {
        if (!out) throw sdpg_error(SDPG_ERR_ARG, "null output pointer");
        *out = nullptr;
        SDPG_CUDA(cudaSetDevice(device));
        auto *h = new sdpg_policy();
        Policy &p = h->p;
        p.device = device;
        try {
            SDPG_CUDA(cudaMalloc(&p.params, kPolParams * sizeof(float)));
            SDPG_CUDA(cudaMalloc(&p.scale, kPolScale * sizeof(float)));
            SDPG_CUDA(cudaMalloc(&p.grad, kPolParams * sizeof(float)));
            SDPG_CUDA(cudaMalloc(&p.m1, kPolParams * sizeof(float)));
            SDPG_CUDA(cudaMalloc(&p.m2, kPolParams * sizeof(float)));
            SDPG_CUDA(cudaMalloc(&p.loss, sizeof(float)));
            std::vector<float> w, sc;
            init_params(w, sc);
            SDPG_CUDA(cudaMemcpy(p.params, w.data(), kPolParams * sizeof(float), cudaMemcpyHostToDevice));
            SDPG_CUDA(cudaMemcpy(p.scale, sc.data(), kPolScale * sizeof(float), cudaMemcpyHostToDevice));
            SDPG_CUDA(cudaMemset(p.grad, 0, kPolParams * sizeof(float)));
            SDPG_CUDA(cudaMemset(p.m1, 0, kPolParams * sizeof(float)));
            SDPG_CUDA(cudaMemset(p.m2, 0, kPolParams * sizeof(float)));
        } catch (...) {
            sdpg_policy_destroy(h);
            throw;
        }
        *out = h;
        return SDPG_OK;
    });
}

void sdpg_policy_destroy(sdpg_policy *h) {
    if (!h) return;
    Policy &p = h->p;
    cudaSetDevice(p.device);
    cudaFree(p.params);
    cudaFree(p.scale);
    cudaFree(p.grad);
    cudaFree(p.m1);
    cudaFree(p.m2);
    cudaFree(p.loss);
    delete h;
}

int sdpg_policy_set(sdpg_policy *h, const float *params, const float *scale) {
    return sdpg_guard([&] {
        Policy &p = get(h);
        if (scale) check_scale(scale);
        if (params) SDPG_CUDA(cudaMemcpy(p.params, params, kPolParams * sizeof(float), cudaMemcpyHostToDevice));
        if (scale) SDPG_CUDA(cudaMemcpy(p.scale, scale, kPolScale * sizeof(float), cudaMemcpyHostToDevice));
        // a new starting point for training: fresh Adam moments
        SDPG_CUDA(cudaMemset(p.m1, 0, kPolParams * sizeof(float)));
        SDPG_CUDA(cudaMemset(p.m2, 0, kPolParams * sizeof(float)));
        p.adam_step = 0;
        return SDPG_OK;
    });
}

int sdpg_policy_get(sdpg_policy *h, float *params, float *scale) {
    return sdpg_guard([&] {
        Policy &p = get(h);
        if (params) SDPG_CUDA(cudaMemcpy(params, p.params, kPolParams * sizeof(float), cudaMemcpyDeviceToHost));
        if (scale) SDPG_CUDA(cudaMemcpy(scale, p.scale, kPolScale * sizeof(float), cudaMemcpyDeviceToHost));
        return SDPG_OK;
    });
}

int sdpg_policy_forward(sdpg_policy *h, const float *x, int count, float *y) {
    return sdpg_guard([&] {
        Policy &p = get(h);
        if (count < 0 || (count > 0 && (!x || !y))) throw sdpg_error(SDPG_ERR_ARG, "bad forward arguments");
        if (count == 0) return SDPG_OK;
        DevFloats dx((size_t)count * kPolIn), dy((size_t)count * kPolOut);
        SDPG_CUDA(cudaMemcpy(dx.p, x, (size_t)count * kPolIn * sizeof(float), cudaMemcpyHostToDevice));
        policy_forward_device(p, dx.p, count, dy.p, 0);
        SDPG_CUDA(cudaMemcpy(y, dy.p, (size_t)count * kPolOut * sizeof(float), cudaMemcpyDeviceToHost));
        return SDPG_OK;
    });
}

int sdpg_policy_gradient(sdpg_policy *h, const float *x, const float *t, const float *mask, int count, float *grad,
                         float *loss) {
    return sdpg_guard([&] {
        Policy &p = get(h);
        if (count <= 0 || !x || !t || !mask || !grad || !loss) throw sdpg_error(SDPG_ERR_ARG, "bad gradient arguments");
        DevFloats dx((size_t)count * kPolIn), dt((size_t)count * kPolOut), dm((size_t)count * kPolOut);
        SDPG_CUDA(cudaMemcpy(dx.p, x, (size_t)count * kPolIn * sizeof(float), cudaMemcpyHostToDevice));
        SDPG_CUDA(cudaMemcpy(dt.p, t, (size_t)count * kPolOut * sizeof(float), cudaMemcpyHostToDevice));
        SDPG_CUDA(cudaMemcpy(dm.p, mask, (size_t)count * kPolOut * sizeof(float), cudaMemcpyHostToDevice));
        SDPG_CUDA(cudaMemset(p.grad, 0, kPolParams * sizeof(float)));
        SDPG_CUDA(cudaMemset(p.loss, 0, sizeof(float)));
        launch(p, dx.p, dt.p, dm.p, nullptr, 0, count, 1.f / count, nullptr, p.grad, p.loss, 0);
        SDPG_CUDA(cudaMemcpy(grad, p.grad, kPolParams * sizeof(float), cudaMemcpyDeviceToHost));
        SDPG_CUDA(cudaMemcpy(loss, p.loss, sizeof(float), cudaMemcpyDeviceToHost));
        SDPG_CUDA(cudaMemset(p.grad, 0, kPolParams * sizeof(float)));
        return SDPG_OK;
    });
}

int sdpg_policy_train(sdpg_policy *h, const float *x, const float *t, const float *mask, int count, int epochs,
                      int batch, float lr, unsigned long long seed, float *epoch_loss) {
    return sdpg_guard([&] {
        Policy &p = get(h);
        if (count <= 0 || epochs < 0 || batch <= 0 || !(lr > 0.f) || !x || !t || !mask)
            throw sdpg_error(SDPG_ERR_ARG, "bad training arguments");
        cudaStream_t s = nullptr;
        SDPG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        try {
            DevFloats dx((size_t)count * kPolIn), dt((size_t)count * kPolOut), dm((size_t)count * kPolOut);
            DevFloats dloss((size_t)std::max(epochs, 1));
            int *dperm = nullptr;
            SDPG_CUDA(cudaMalloc(&dperm, (size_t)count * sizeof(int)));
            std::unique_ptr<int, decltype(&cudaFree)> perm_guard(dperm, &cudaFree);
            SDPG_CUDA(cudaMemcpyAsync(dx.p, x, (size_t)count * kPolIn * sizeof(float), cudaMemcpyHostToDevice, s));
            SDPG_CUDA(cudaMemcpyAsync(dt.p, t, (size_t)count * kPolOut * sizeof(float), cudaMemcpyHostToDevice, s));
            SDPG_CUDA(cudaMemcpyAsync(dm.p, mask, (size_t)count * kPolOut * sizeof(float), cudaMemcpyHostToDevice, s));
            SDPG_CUDA(cudaMemsetAsync(dloss.p, 0, (size_t)std::max(epochs, 1) * sizeof(float), s));
            SDPG_CUDA(cudaMemsetAsync(p.grad, 0, kPolParams * sizeof(float), s));
            std::vector<int> perm(count);
            for (int i = 0; i < count; ++i) perm[i] = i;
            std::mt19937_64 g(seed);
            const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
            for (int e = 0; e < epochs; ++e) {
                // Fisher-Yates with an explicit bounded draw, identical on every platform
                for (int i = count - 1; i > 0; --i) std::swap(perm[i], perm[(size_t)(g() % (unsigned long long)(i + 1))]);
                SDPG_CUDA(cudaMemcpyAsync(dperm, perm.data(), (size_t)count * sizeof(int), cudaMemcpyHostToDevice, s));
                const int nbatch = (count + batch - 1) / batch;
                for (int b0 = 0; b0 < count; b0 += batch) {
                    const int bs = std::min(batch, count - b0);
                    launch(p, dx.p, dt.p, dm.p, dperm, b0, bs, 1.f / bs, nullptr, p.grad, dloss.p + e, s);
                    ++p.adam_step;
                    const float bc1 = (float)(1.0 - pow((double)b1, (double)p.adam_step));
                    const float bc2 = (float)(1.0 - pow((double)b2, (double)p.adam_step));
                    SDPG_KT_BEGIN(s);
                    policy_adam_kernel<<<(kPolParams + 255) / 256, 256, 0, s>>>(p.params, p.grad, p.m1, p.m2,
                                                                               kPolParams, lr, b1, b2, eps, bc1, bc2);
                    SDPG_CHECK_LAUNCH_KT("policy_adam_kernel", s);
                }
                // the host permutation is rewritten next epoch: wait for its copy
                SDPG_CUDA(cudaStreamSynchronize(s));
            }
            if (epoch_loss && epochs > 0) {
                std::vector<float> l(epochs);
                SDPG_CUDA(cudaMemcpyAsync(l.data(), dloss.p, epochs * sizeof(float), cudaMemcpyDeviceToHost, s));
                SDPG_CUDA(cudaStreamSynchronize(s));
                const int nbatch = (count + batch - 1) / batch;  // the epoch loss: mean of the batch losses
                for (int e = 0; e < epochs; ++e) epoch_loss[e] = l[e] / nbatch;
            }
            SDPG_CUDA(cudaStreamSynchronize(s));
        } catch (...) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
            throw;
        }
        SDPG_CUDA(cudaStreamDestroy(s));
        return SDPG_OK;
    });
}

}  // extern "C"
