// gbs_mlp.cu -- training of the bucket-width controller (include/gbsssp.h,
// "Controller training"): FP32 MLP 16 -> 64 -> 64 -> 2 (ReLU) in the
// parameter layout of gbs_internal.cuh (kMlp*), hand-written kernels:
//
//   k_mlp_grad   one CTA of 64 threads per chunk of samples: forward pass,
//                loss and backward pass per sample, weight gradients summed
//                in shared memory (thread o owns column o of every matrix,
//                so no two threads write one sum) and added to the global
//                gradient once per CTA
//   k_mlp_adam   one thread per parameter (bias-corrected Adam)
//   k_mlp_fwd    inference for a batch (evaluation)
//
// Loss of sample i with weight w_i, outputs y0 (log2 of the bucket-width
// scale) and y1 (split logit), targets t0 and t1 in {0, 1}:
//   L = sum_i w_i [ (y0 - t0)^2 + BCE(sigmoid(y1), t1) ] / sum_i w_i
// The layers (16x64, 64x64) are far too small per sample to fill a
// tensor-core tile, and a batch is a few MFLOP, so plain FP32 FMAs are used.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "gbs_host.hpp"

using namespace gbs;

struct gbs_mlp {
    float *d_p = nullptr;      // kMlpFloats: normaliser + parameters
    float *d_g = nullptr;      // kMlpParams gradient
    float *d_m = nullptr, *d_v = nullptr;   // Adam moments
    float *d_x = nullptr, *d_t = nullptr, *d_w = nullptr;   // data
    uint32_t *d_idx = nullptr; // sample order
    double *d_loss = nullptr;  // weighted loss sum of the last batch
    std::vector<float> w_host; // sample weights (batch weight sums)
    uint32_t n = 0;
    uint32_t step = 0;
    cudaStream_t stream = nullptr;
};

namespace {

constexpr int kMlpThreads = kHid;   // 64

__device__ __forceinline__ float sigmoid_f(float z) { return 1.f / (1.f + expf(-z)); }

// Forward + backward over samples idx[first + k], k in [0, count), a chunk of
// consecutive k per CTA.
__global__ void __launch_bounds__(kMlpThreads) k_mlp_grad(const float *__restrict__ P, const float *__restrict__ X,
                                                          const float *__restrict__ T, const float *__restrict__ Wt,
                                                          const uint32_t *__restrict__ idx, uint32_t first,
                                                          uint32_t count, uint32_t chunk, float inv_wsum,
                                                          float *__restrict__ G, double *__restrict__ loss) {
    __shared__ float sW1[kFeat * kHid], sW2[kHid * kHid], sW3[kHid * 2];
    __shared__ float gW1[kFeat * kHid], gW2[kHid * kHid], gW3[kHid * 2], gb1[kHid], gb2[kHid], gb3[2];
    __shared__ float xn[kFeat], h1[kHid], h2[kHid], dh2[kHid], dy[2];
    __shared__ double s_loss;
    const int o = threadIdx.x;
    for (int i = o; i < kFeat * kHid; i += kMlpThreads) {
        sW1[i] = P[kMlpW1 + i];
        gW1[i] = 0.f;
    }
    for (int i = o; i < kHid * kHid; i += kMlpThreads) {
        sW2[i] = P[kMlpW2 + i];
        gW2[i] = 0.f;
    }
    for (int i = o; i < kHid * 2; i += kMlpThreads) {
        sW3[i] = P[kMlpW3 + i];
        gW3[i] = 0.f;
    }
    gb1[o] = 0.f;
    gb2[o] = 0.f;
    if (o < 2) gb3[o] = 0.f;
    if (o == 0) s_loss = 0.0;
    const float b1 = P[kMlpB1 + o], b2 = P[kMlpB2 + o];
    __syncthreads();
    const uint32_t s0 = blockIdx.x * chunk;
    const uint32_t s1 = min(count, s0 + chunk);
    for (uint32_t k = s0; k < s1; ++k) {
        const uint32_t i = idx[first + k];
        if (o < kFeat) xn[o] = (X[(size_t)i * kFeat + o] - P[o]) / P[kFeat + o];
        __syncthreads();
        // forward
        float a1 = b1;
#pragma unroll
        for (int f = 0; f < kFeat; ++f) a1 = fmaf(xn[f], sW1[f * kHid + o], a1);
        h1[o] = fmaxf(a1, 0.f);
        __syncthreads();
        float a2 = b2;
#pragma unroll 16
        for (int f = 0; f < kHid; ++f) a2 = fmaf(h1[f], sW2[f * kHid + o], a2);
        h2[o] = fmaxf(a2, 0.f);
        __syncthreads();
        if (o < 2) {
            float y = P[kMlpB3 + o];
            for (int f = 0; f < kHid; ++f) y = fmaf(h2[f], sW3[f * 2 + o], y);
            const float w = Wt[i] * inv_wsum;
            const float t = T[(size_t)i * 2 + o];
            float l, d;
            if (o == 0) {
                const float e = y - t;
                l = e * e;
                d = 2.f * e;
            } else {
                // BCE with logits: max(y, 0) - y t + log(1 + exp(-|y|))
                l = fmaxf(y, 0.f) - y * t + log1pf(expf(-fabsf(y)));
                d = sigmoid_f(y) - t;
            }
            dy[o] = w * d;
            atomicAdd(&s_loss, (double)(w * l));
        }
        __syncthreads();
        // backward: output layer (thread o owns row o of W3)
        const float h2o = h2[o];
        gW3[o * 2] += h2o * dy[0];
        gW3[o * 2 + 1] += h2o * dy[1];
        if (o < 2) gb3[o] += dy[o];
        const float g2 = (h2o > 0.f) ? (sW3[o * 2] * dy[0] + sW3[o * 2 + 1] * dy[1]) : 0.f;
        dh2[o] = g2;
        gb2[o] += g2;
        __syncthreads();
        // W2 column o, and the gradient reaching h1[o] (row o of W2)
#pragma unroll 16
        for (int f = 0; f < kHid; ++f) gW2[f * kHid + o] += h1[f] * g2;
        float g1 = 0.f;
#pragma unroll 16
        for (int f = 0; f < kHid; ++f) g1 = fmaf(sW2[o * kHid + f], dh2[f], g1);
        g1 = (h1[o] > 0.f) ? g1 : 0.f;
        gb1[o] += g1;
#pragma unroll
        for (int f = 0; f < kFeat; ++f) gW1[f * kHid + o] += xn[f] * g1;
        __syncthreads();
    }
    // one global add per parameter per CTA
    for (int i = o; i < kFeat * kHid; i += kMlpThreads) atomicAdd(&G[kMlpW1 - 2 * kFeat + i], gW1[i]);
    atomicAdd(&G[kMlpB1 - 2 * kFeat + o], gb1[o]);
    for (int i = o; i < kHid * kHid; i += kMlpThreads) atomicAdd(&G[kMlpW2 - 2 * kFeat + i], gW2[i]);
    atomicAdd(&G[kMlpB2 - 2 * kFeat + o], gb2[o]);
    for (int i = o; i < kHid * 2; i += kMlpThreads) atomicAdd(&G[kMlpW3 - 2 * kFeat + i], gW3[i]);
    if (o < 2) atomicAdd(&G[kMlpB3 - 2 * kFeat + o], gb3[o]);
    if (o == 0) atomicAdd(loss, s_loss);
}

__global__ void k_mlp_adam(float *__restrict__ P, const float *__restrict__ G, float *__restrict__ M,
                           float *__restrict__ V, float lr, float beta1, float beta2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    const float g = G[i];
    const float m = beta1 * M[i] + (1.f - beta1) * g;
    const float v = beta2 * V[i] + (1.f - beta2) * g * g;
    M[i] = m;
    V[i] = v;
    P[2 * kFeat + i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

__global__ void k_mlp_fwd(const float *__restrict__ P, const float *__restrict__ X, uint32_t n,
                          float *__restrict__ Y) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float xn[kFeat], h1[kHid];
#pragma unroll
    for (int f = 0; f < kFeat; ++f) xn[f] = (X[(size_t)i * kFeat + f] - P[f]) / P[kFeat + f];
    for (int o = 0; o < kHid; ++o) {
        float a = P[kMlpB1 + o];
#pragma unroll
        for (int f = 0; f < kFeat; ++f) a = fmaf(xn[f], P[kMlpW1 + f * kHid + o], a);
        h1[o] = fmaxf(a, 0.f);
    }
    float y0 = P[kMlpB3], y1 = P[kMlpB3 + 1];
    for (int o = 0; o < kHid; ++o) {
        float a = P[kMlpB2 + o];
        for (int f = 0; f < kHid; ++f) a = fmaf(h1[f], P[kMlpW2 + f * kHid + o], a);
        a = fmaxf(a, 0.f);
        y0 = fmaf(a, P[kMlpW3 + 2 * o], y0);
        y1 = fmaf(a, P[kMlpW3 + 2 * o + 1], y1);
    }
    Y[2 * (size_t)i] = y0;
    Y[2 * (size_t)i + 1] = y1;
}

void free_mlp(gbs_mlp *m) {
    if (!m) return;
    cudaFree(m->d_p); cudaFree(m->d_g); cudaFree(m->d_m); cudaFree(m->d_v);
    cudaFree(m->d_x); cudaFree(m->d_t); cudaFree(m->d_w); cudaFree(m->d_idx); cudaFree(m->d_loss);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

// Gradient (into d_g, zeroed first) and loss over samples idx[first, first +
// count); idx is the host copy of the order held on the device.
gbs_status grad_range(gbs_mlp *m, const std::vector<uint32_t> &idx, uint32_t first, uint32_t count,
                      double *loss) {
    if (count == 0) return fail(GBS_ERR_INVALID_ARG, "empty batch");
    double wsum = 0.0;
    for (uint32_t k = first; k < first + count; ++k) wsum += m->w_host[idx[k]];
    if (!(wsum > 0)) return fail(GBS_ERR_INVALID_ARG, "batch weights sum to zero");
    GBS_CUDA(cudaMemsetAsync(m->d_g, 0, sizeof(float) * kMlpParams, m->stream));
    GBS_CUDA(cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->stream));
    const uint32_t chunk = 16;
    const uint32_t blocks = (count + chunk - 1) / chunk;
    k_mlp_grad<<<blocks, kMlpThreads, 0, m->stream>>>(m->d_p, m->d_x, m->d_t, m->d_w, m->d_idx, first, count,
                                                       chunk, (float)(1.0 / wsum), m->d_g, m->d_loss);
    GBS_CUDA(cudaGetLastError());
    if (loss) {
        GBS_CUDA(cudaMemcpyAsync(loss, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
        GBS_CUDA(cudaStreamSynchronize(m->stream));
    }
    return GBS_OK;
}

gbs_status adam_step(gbs_mlp *m, float lr, float beta1, float beta2, float eps) {
    m->step += 1;
    const float c1 = 1.f - std::pow(beta1, (float)m->step);
    const float c2 = 1.f - std::pow(beta2, (float)m->step);
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, m->stream>>>(m->d_p, m->d_g, m->d_m, m->d_v, lr, beta1, beta2,
                                                               eps, c1, c2);
    GBS_CUDA(cudaGetLastError());
    return GBS_OK;
}

}  // namespace

extern "C" {

gbs_status gbs_mlp_create(gbs_mlp **out) {
    if (!out) return fail(GBS_ERR_INVALID_ARG, "out is NULL");
    gbs_mlp *m = new gbs_mlp();
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_p, sizeof(float) * kMlpFloats)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_g, sizeof(float) * kMlpParams)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_m, sizeof(float) * kMlpParams)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_v, sizeof(float) * kMlpParams)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_loss, sizeof(double))) != cudaSuccess ||
        (e = cudaMemset(m->d_p, 0, sizeof(float) * kMlpFloats)) != cudaSuccess ||
        (e = cudaMemset(m->d_g, 0, sizeof(float) * kMlpParams)) != cudaSuccess ||
        (e = cudaMemset(m->d_m, 0, sizeof(float) * kMlpParams)) != cudaSuccess ||
        (e = cudaMemset(m->d_v, 0, sizeof(float) * kMlpParams)) != cudaSuccess) {
        free_mlp(m);
        return fail(e == cudaErrorMemoryAllocation ? GBS_ERR_NO_MEMORY : GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = m;
    return GBS_OK;
}

gbs_status gbs_mlp_destroy(gbs_mlp *m) {
    if (!m) return fail(GBS_ERR_INVALID_ARG, "mlp is NULL");
    cudaStreamSynchronize(m->stream);
    free_mlp(m);
    return GBS_OK;
}

gbs_status gbs_mlp_set_params(gbs_mlp *m, const float *params) {
    if (!m || !params) return fail(GBS_ERR_INVALID_ARG, "NULL argument");
    GBS_CUDA(cudaMemcpy(m->d_p, params, sizeof(float) * kMlpFloats, cudaMemcpyHostToDevice));
    GBS_CUDA(cudaMemset(m->d_m, 0, sizeof(float) * kMlpParams));
    GBS_CUDA(cudaMemset(m->d_v, 0, sizeof(float) * kMlpParams));
    m->step = 0;
    return GBS_OK;
}

gbs_status gbs_mlp_get_params(gbs_mlp *m, float *params) {
    if (!m || !params) return fail(GBS_ERR_INVALID_ARG, "NULL argument");
    GBS_CUDA(cudaStreamSynchronize(m->stream));
    GBS_CUDA(cudaMemcpy(params, m->d_p, sizeof(float) * kMlpFloats, cudaMemcpyDeviceToHost));
    return GBS_OK;
}

gbs_status gbs_mlp_set_data(gbs_mlp *m, const float *x, const float *t, const float *w, uint32_t n) {
    if (!m || !x || !t || n == 0) return fail(GBS_ERR_INVALID_ARG, "NULL argument or no samples");
    cudaFree(m->d_x); cudaFree(m->d_t); cudaFree(m->d_w); cudaFree(m->d_idx);
    m->d_x = m->d_t = m->d_w = nullptr;
    m->d_idx = nullptr;
    m->n = n;
    GBS_CUDA(cudaMalloc(&m->d_x, sizeof(float) * kFeat * n));
    GBS_CUDA(cudaMalloc(&m->d_t, sizeof(float) * 2 * n));
    GBS_CUDA(cudaMalloc(&m->d_w, sizeof(float) * n));
    GBS_CUDA(cudaMalloc(&m->d_idx, sizeof(uint32_t) * n));
    GBS_CUDA(cudaMemcpy(m->d_x, x, sizeof(float) * kFeat * n, cudaMemcpyHostToDevice));
    GBS_CUDA(cudaMemcpy(m->d_t, t, sizeof(float) * 2 * n, cudaMemcpyHostToDevice));
    if (w) m->w_host.assign(w, w + n);
    else m->w_host.assign(n, 1.f);
    GBS_CUDA(cudaMemcpy(m->d_w, m->w_host.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    GBS_CUDA(cudaMemcpy(m->d_idx, idx.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    return GBS_OK;
}

gbs_status gbs_mlp_loss_grad(gbs_mlp *m, uint32_t first, uint32_t count, double *loss, float *grad) {
    if (!m || !m->n) return fail(GBS_ERR_INVALID_ARG, "no data");
    if ((uint64_t)first + count > m->n) return fail(GBS_ERR_INVALID_ARG, "sample range out of bounds");
    // samples in stored order for this call
    std::vector<uint32_t> idx(m->n);
    std::iota(idx.begin(), idx.end(), 0u);
    GBS_CUDA(cudaMemcpy(m->d_idx, idx.data(), sizeof(uint32_t) * m->n, cudaMemcpyHostToDevice));
    gbs_status st = grad_range(m, idx, first, count, loss);
    if (st != GBS_OK) return st;
    if (grad) {
        GBS_CUDA(cudaMemcpyAsync(grad, m->d_g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->stream));
        GBS_CUDA(cudaStreamSynchronize(m->stream));
    }
    return GBS_OK;
}

gbs_status gbs_mlp_adam(gbs_mlp *m, float lr, float beta1, float beta2, float eps) {
    if (!m) return fail(GBS_ERR_INVALID_ARG, "mlp is NULL");
    gbs_status st = adam_step(m, lr, beta1, beta2, eps);
    if (st != GBS_OK) return st;
    GBS_CUDA(cudaStreamSynchronize(m->stream));
    return GBS_OK;
}

gbs_status gbs_mlp_train(gbs_mlp *m, uint32_t epochs, uint32_t batch, float lr, uint64_t seed, double *epoch_loss) {
    if (!m || !m->n || batch == 0) return fail(GBS_ERR_INVALID_ARG, "no data or batch 0");
    std::mt19937_64 rng(seed);
    std::vector<uint32_t> idx(m->n);
    std::iota(idx.begin(), idx.end(), 0u);
    for (uint32_t ep = 0; ep < epochs; ++ep) {
        std::shuffle(idx.begin(), idx.end(), rng);
        GBS_CUDA(cudaMemcpyAsync(m->d_idx, idx.data(), sizeof(uint32_t) * m->n, cudaMemcpyHostToDevice, m->stream));
        double total = 0.0;
        uint32_t nb = 0;
        for (uint32_t b = 0; b < m->n; b += batch) {
            const uint32_t cnt = std::min(batch, m->n - b);
            double l = 0.0;
            gbs_status st = grad_range(m, idx, b, cnt, &l);
            if (st != GBS_OK) return st;
            st = adam_step(m, lr, 0.9f, 0.999f, 1e-8f);
            if (st != GBS_OK) return st;
            total += l;
            ++nb;
        }
        if (epoch_loss) epoch_loss[ep] = nb ? total / nb : 0.0;
    }
    GBS_CUDA(cudaStreamSynchronize(m->stream));
    return GBS_OK;
}

gbs_status gbs_mlp_predict(gbs_mlp *m, const float *x, uint32_t n, float *y) {
    if (!m || !x || !y) return fail(GBS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return GBS_OK;
    float *dx = nullptr, *dy = nullptr;
    GBS_CUDA(cudaMalloc(&dx, sizeof(float) * kFeat * n));
    cudaError_t e = cudaMalloc(&dy, sizeof(float) * 2 * n);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(float) * kFeat * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_mlp_fwd<<<(n + 127) / 128, 128, 0, m->stream>>>(m->d_p, dx, n, dy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return fail(GBS_ERR_CUDA, cudaGetErrorString(e));
    return GBS_OK;
}

}  // extern "C"
