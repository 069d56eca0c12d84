// The learned parameter proposal: a fully connected FP32 network with three hidden
// layers of 64 tanh units that maps six interior-point features to two outputs,
//   in:  log10 mu, log10 |primal residual|_max, log10 |dual residual|_max,
//        previous primal step length, previous dual step length,
//        the centering value of the Mehrotra rule at this iteration
//   out: log10 lambdaStar (read at the initial point), beta (the corrector's centering).
// Inputs are standardised and outputs de-standardised with fixed per-feature shifts
// and scales that the trainer sets.  There is no counterpart in the reference solver,
// whose lambdaStar and betaStar/betaBar are constants of param.sdpa.
#pragma once
#include <cuda_runtime.h>

namespace sdpg {

constexpr int kPolIn = 6;
constexpr int kPolH = 64;
constexpr int kPolOut = 2;
// flat parameter layout: W1[64][6] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[2][64] b4[2]
constexpr int kPolW1 = 0;
constexpr int kPolB1 = kPolW1 + kPolH * kPolIn;
constexpr int kPolW2 = kPolB1 + kPolH;
constexpr int kPolB2 = kPolW2 + kPolH * kPolH;
constexpr int kPolW3 = kPolB2 + kPolH;
constexpr int kPolB3 = kPolW3 + kPolH * kPolH;
constexpr int kPolW4 = kPolB3 + kPolH;
constexpr int kPolB4 = kPolW4 + kPolOut * kPolH;
constexpr int kPolParams = kPolB4 + kPolOut;  // 8898
// scaling: x_mean[6] x_std[6] y_mean[2] y_std[2]
constexpr int kPolScale = 2 * kPolIn + 2 * kPolOut;

struct Policy {
    int device = 0;
    float *params = nullptr;  // device, kPolParams
    float *scale = nullptr;   // device, kPolScale
    float *grad = nullptr, *m1 = nullptr, *m2 = nullptr, *loss = nullptr;
    long long adam_step = 0;
};

// y (device, count x 2, de-standardised) = network(x (device, count x 6)) on stream s.
void policy_forward_device(const Policy &p, const float *x, int count, float *y, cudaStream_t s);

}  // namespace sdpg

// the C-ABI handle (sdpg.h)
struct sdpg_policy {
    sdpg::Policy p;
};
