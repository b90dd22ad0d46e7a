// mlp.cu -- the learned parameter selector's network: an FP32 multilayer
// perceptron 8 -> 64 -> 64 -> 4 with tanh hidden units, its inference, its
// mean-squared-error gradient and an Adam step, as hand-written kernels.
//
// No counterpart in the reference (which picks xi, M, P and the cutoff from
// analytic error estimates only).  Parameters live in one FP32 vector:
//   W1 [64 x 8], b1 [64], W2 [64 x 64], b2 [64], W3 [4 x 64], b3 [4]
// (row-major, y = W x + b).  All entries take device pointers and a stream.
//
// Training step over n samples X [n x 8] with targets T [n x 4] and
// per-sample weights s [n] (null: 1):
//   loss = (1/n) sum_i s_i |y_i - t_i|^2
// k_mlp_forward keeps H1, H2 (tanh outputs); k_mlp_delta forms the output and
// hidden deltas per sample (D3 = 2 s (y - t) / n, D2 = (W3^T D3)(1 - H2^2),
// D1 = (W2^T D2)(1 - H1^2)); k_mlp_wgrad reduces the outer products over the
// samples, one thread per parameter (deterministic: fixed summation order).
#include <cmath>

#include "fte_internal.cuh"

namespace {
constexpr int kIn = FTE_MLP_IN, kH = FTE_MLP_HIDDEN, kOut = FTE_MLP_OUT;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kOut * kH, kParams = oB3 + kOut;
static_assert(kParams == FTE_MLP_PARAMS, "parameter layout");

constexpr int kThreads = 128;

// forward pass, one sample per thread; parameters staged in shared memory
__global__ void __launch_bounds__(kThreads) k_mlp_forward(const float* __restrict__ prm, const float* __restrict__ X,
                                                         int n, float* __restrict__ Y, float* __restrict__ H1,
                                                         float* __restrict__ H2) {
    __shared__ float w[kParams];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = prm[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[kIn], h1[kH], h2[kH];
#pragma unroll
    for (int i = 0; i < kIn; i++) x[i] = X[(size_t)s * kIn + i];
#pragma unroll 4
    for (int j = 0; j < kH; j++) {
        float a = w[oB1 + j];
#pragma unroll
        for (int i = 0; i < kIn; i++) a = fmaf(w[oW1 + j * kIn + i], x[i], a);
        h1[j] = tanhf(a);
    }
#pragma unroll 2
    for (int j = 0; j < kH; j++) {
        float a = w[oB2 + j];
#pragma unroll
        for (int i = 0; i < kH; i++) a = fmaf(w[oW2 + j * kH + i], h1[i], a);
        h2[j] = tanhf(a);
    }
#pragma unroll
    for (int o = 0; o < kOut; o++) {
        float a = w[oB3 + o];
#pragma unroll
        for (int i = 0; i < kH; i++) a = fmaf(w[oW3 + o * kH + i], h2[i], a);
        Y[(size_t)s * kOut + o] = a;
    }
    if (H1) {
        for (int j = 0; j < kH; j++) H1[(size_t)s * kH + j] = h1[j];
        for (int j = 0; j < kH; j++) H2[(size_t)s * kH + j] = h2[j];
    }
}

// per-sample deltas and weighted squared error
__global__ void __launch_bounds__(kThreads) k_mlp_delta(const float* __restrict__ prm, const float* __restrict__ Y,
                                                       const float* __restrict__ T, const float* __restrict__ sw,
                                                       int n, float inv_n, const float* __restrict__ H1,
                                                       const float* __restrict__ H2, float* __restrict__ D3,
                                                       float* __restrict__ D2, float* __restrict__ D1,
                                                       float* __restrict__ err) {
    __shared__ float w[kParams];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = prm[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float ws = (sw ? sw[s] : 1.0f) * inv_n;
    float d3[kOut], d2[kH];
    float e = 0.f;
#pragma unroll
    for (int o = 0; o < kOut; o++) {
        float r = Y[(size_t)s * kOut + o] - T[(size_t)s * kOut + o];
        e = fmaf(r, r, e);
        d3[o] = 2.0f * ws * r;
        D3[(size_t)s * kOut + o] = d3[o];
    }
    err[s] = e * ws;
    for (int i = 0; i < kH; i++) {
        float a = 0.f;
#pragma unroll
        for (int o = 0; o < kOut; o++) a = fmaf(w[oW3 + o * kH + i], d3[o], a);
        float h = H2[(size_t)s * kH + i];
        d2[i] = a * (1.0f - h * h);
        D2[(size_t)s * kH + i] = d2[i];
    }
    for (int i = 0; i < kH; i++) {
        float a = 0.f;
#pragma unroll 8
        for (int j = 0; j < kH; j++) a = fmaf(w[oW2 + j * kH + i], d2[j], a);
        float h = H1[(size_t)s * kH + i];
        D1[(size_t)s * kH + i] = a * (1.0f - h * h);
    }
}

// gradient of every parameter: sum over samples of delta x input
__global__ void k_mlp_wgrad(const float* __restrict__ X, const float* __restrict__ H1, const float* __restrict__ H2,
                            const float* __restrict__ D1, const float* __restrict__ D2, const float* __restrict__ D3,
                            const float* __restrict__ err, int n, float* __restrict__ grad, float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kParams) return;
    float acc = 0.f;
    if (p == kParams) {  // the loss
        for (int s = 0; s < n; s++) acc += err[s];
        *loss = acc;
        return;
    }
    const float *d, *a;
    int dstride, astride, di, ai;
    if (p < oB1) {
        di = (p - oW1) / kIn, ai = (p - oW1) % kIn;
        d = D1, dstride = kH, a = X, astride = kIn;
    } else if (p < oW2) {
        di = p - oB1, ai = -1;
        d = D1, dstride = kH, a = nullptr, astride = 0;
    } else if (p < oB2) {
        di = (p - oW2) / kH, ai = (p - oW2) % kH;
        d = D2, dstride = kH, a = H1, astride = kH;
    } else if (p < oW3) {
        di = p - oB2, ai = -1;
        d = D2, dstride = kH, a = nullptr, astride = 0;
    } else if (p < oB3) {
        di = (p - oW3) / kH, ai = (p - oW3) % kH;
        d = D3, dstride = kOut, a = H2, astride = kH;
    } else {
        di = p - oB3, ai = -1;
        d = D3, dstride = kOut, a = nullptr, astride = 0;
    }
    for (int s = 0; s < n; s++) {
        float dv = d[(size_t)s * dstride + di];
        acc = a ? fmaf(dv, a[(size_t)s * astride + ai], acc) : acc + dv;
    }
    grad[p] = acc;
}

// Adam (Kingma & Ba 2015) with bias correction
__global__ void k_mlp_adam(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                           float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / c1, vh = vi / c2;
    prm[i] -= lr * mh / (sqrtf(vh) + eps);
}

int launch_check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fte_set_error("%s: %s", what, cudaGetErrorString(e));
        return FTE_ERR_CUDA;
    }
    return FTE_OK;
}
}  // namespace

extern "C" int fte_mlp_param_count(void) { return kParams; }

extern "C" size_t fte_mlp_scratch_floats(int n) {
    // H1, H2, D1, D2 (n x 64 each), Y, D3 (n x 4 each), err (n)
    return (size_t)n * (4 * kH + 2 * kOut + 1);
}

extern "C" int fte_mlp_forward(const float* params, const float* X, int n, float* Y, void* stream) {
    if (n < 0 || (n > 0 && (!params || !X || !Y))) {
        fte_set_error("fte_mlp_forward: bad arguments");
        return FTE_ERR_INVALID;
    }
    if (n == 0) return FTE_OK;
    k_mlp_forward<<<(n + kThreads - 1) / kThreads, kThreads, 0, (cudaStream_t)stream>>>(params, X, n, Y, nullptr,
                                                                                       nullptr);
    return launch_check("fte_mlp_forward");
}

extern "C" int fte_mlp_loss_grad(const float* params, const float* X, const float* T, const float* weights, int n,
                                 float* scratch, float* grad, float* loss, void* stream) {
    if (n <= 0 || !params || !X || !T || !scratch || !grad || !loss) {
        fte_set_error("fte_mlp_loss_grad: bad arguments");
        return FTE_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    float* H1 = scratch;
    float* H2 = H1 + (size_t)n * kH;
    float* D1 = H2 + (size_t)n * kH;
    float* D2 = D1 + (size_t)n * kH;
    float* Y = D2 + (size_t)n * kH;
    float* D3 = Y + (size_t)n * kOut;
    float* err = D3 + (size_t)n * kOut;
    const float inv = 1.0f / (float)n;
    const int nb = (n + kThreads - 1) / kThreads;
    k_mlp_forward<<<nb, kThreads, 0, st>>>(params, X, n, Y, H1, H2);
    FTE_TRY(launch_check("fte_mlp_loss_grad forward"));
    k_mlp_delta<<<nb, kThreads, 0, st>>>(params, Y, T, weights, n, inv, H1, H2, D3, D2, D1, err);
    FTE_TRY(launch_check("fte_mlp_loss_grad delta"));
    k_mlp_wgrad<<<(kParams + 1 + 127) / 128, 128, 0, st>>>(X, H1, H2, D1, D2, D3, err, n, grad, loss);
    return launch_check("fte_mlp_loss_grad wgrad");
}

extern "C" int fte_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                            float beta2, float eps, void* stream) {
    if (!params || !grad || !m || !v || step < 1) {
        fte_set_error("fte_mlp_adam: bad arguments");
        return FTE_ERR_INVALID;
    }
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_mlp_adam<<<(kParams + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, kParams, lr, beta1, beta2,
                                                                        eps, c1, c2);
    return launch_check("fte_mlp_adam");
}
