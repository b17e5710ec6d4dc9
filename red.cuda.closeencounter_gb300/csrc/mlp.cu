// mlp.cu -- the learned step-size proposer: an 8 -> 64 -> 64 -> 1 perceptron with SiLU
// activations, BF16 weights and FP32 accumulation, trained on the GPU by the kernels below
// (forward, backward, AdamW) from the attempt logs the ensemble integrator writes.
//
// Not in the reference (the reference has no learned component).  Inputs are standardised
// features of a disk at the start of a step; the output is log(ideal step / last ideal step).
//
// Parameter vector (FP32 master copy; the forward passes read its BF16 image):
//   W1[64][8] b1[64] W2[64][64] b2[64] w3[64] b3
// Training: a CTA owns a tile of MLP_TB samples; activations live in shared memory, the
// matrix products are plain FP32 FMA loops (the network has 4.8k weights -- far too small
// for the tensor cores to matter), and each CTA adds its partial gradient to a global FP32
// buffer with atomics.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "../../include/redgb.h"
#include "common.cuh"
#include "mlp.h"

namespace redgb {
int set_error(int code, const std::string& msg);

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// FP32 master -> BF16 image
__global__ void mlp_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

__device__ __forceinline__ float bf(const __nv_bfloat16* w, int i) { return __bfloat162float(w[i]); }

// Forward (and optionally backward) of a tile of samples.  x: n x 8 (already
// standardised), y: targets (training) ; out: predictions; grad: += dL/dw (FP32).
template <bool TRAIN>
__global__ void __launch_bounds__(256) mlp_tile_kernel(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ x,
                                                      const float* __restrict__ y, const int* __restrict__ index, int n,
                                                      float inv_batch, float* __restrict__ out,
                                                      float* __restrict__ grad, float* __restrict__ loss)
{
    constexpr int H = MLP_HIDDEN, I = MLP_IN, TB = MLP_TB;
    __shared__ float X[TB][I];
    __shared__ float Z1[TB][H + 1];
    __shared__ float Z2[TB][H + 1];
    __shared__ float D[TB];   // dL/dy per sample
    __shared__ float W2s[H][H + 1];
    const int t = threadIdx.x;
    const int s0 = blockIdx.x * TB;
    for (int k = t; k < TB * I; k += blockDim.x) {
        const int s = k / I, f = k % I;
        const int g = s0 + s;
        X[s][f] = g < n ? x[(size_t)(index ? index[g] : g) * I + f] : 0.0f;
    }
    for (int k = t; k < H * H; k += blockDim.x) W2s[k / H][k % H] = bf(wb, MLP_OFF_W2 + k);
    __syncthreads();
    // layer 1: Z1 = X W1^T + b1
    for (int k = t; k < TB * H; k += blockDim.x) {
        const int s = k / H, u = k % H;
        float z = bf(wb, MLP_OFF_B1 + u);
#pragma unroll
        for (int f = 0; f < I; f++) z = fmaf(bf(wb, MLP_OFF_W1 + u * I + f), X[s][f], z);
        Z1[s][u] = z;
    }
    __syncthreads();
    // layer 2: Z2 = silu(Z1) W2^T + b2
    for (int k = t; k < TB * H; k += blockDim.x) {
        const int s = k / H, u = k % H;
        float z = bf(wb, MLP_OFF_B2 + u);
        for (int v = 0; v < H; v++) z = fmaf(W2s[u][v], silu(Z1[s][v]), z);
        Z2[s][u] = z;
    }
    __syncthreads();
    // output: y = w3 . silu(Z2) + b3
    for (int s = t; s < TB; s += blockDim.x) {
        float o = bf(wb, MLP_OFF_B3);
        for (int u = 0; u < H; u++) o = fmaf(bf(wb, MLP_OFF_W3 + u), silu(Z2[s][u]), o);
        const int g = s0 + s;
        if (g < n) {
            if (out) out[g] = o;
            if (TRAIN) {
                const float r = o - y[index ? index[g] : g];
                D[s] = 2.0f * r * inv_batch;
                atomicAdd(loss, r * r * inv_batch);
            }
        } else {
            D[s] = 0.0f;
        }
    }
    if (!TRAIN) return;
    __syncthreads();
    // backward.  dw3 = sum_s D_s silu(Z2_s); db3 = sum_s D_s
    for (int u = t; u < H; u += blockDim.x) {
        float g3 = 0.0f;
        for (int s = 0; s < TB; s++) g3 = fmaf(D[s], silu(Z2[s][u]), g3);
        atomicAdd(&grad[MLP_OFF_W3 + u], g3);
    }
    if (t == 0) {
        float gb = 0.0f;
        for (int s = 0; s < TB; s++) gb += D[s];
        atomicAdd(&grad[MLP_OFF_B3], gb);
    }
    __syncthreads();
    // dZ2 = D w3 * silu'(Z2)  (overwrite Z2 with dZ2 after keeping silu(Z1) available)
    for (int k = t; k < TB * H; k += blockDim.x) {
        const int s = k / H, u = k % H;
        Z2[s][u] = D[s] * bf(wb, MLP_OFF_W3 + u) * dsilu(Z2[s][u]);
    }
    __syncthreads();
    // dW2[u][v] = sum_s dZ2[s][u] silu(Z1[s][v]); db2[u] = sum_s dZ2[s][u]
    for (int k = t; k < H * H; k += blockDim.x) {
        const int u = k / H, v = k % H;
        float g = 0.0f;
        for (int s = 0; s < TB; s++) g = fmaf(Z2[s][u], silu(Z1[s][v]), g);
        atomicAdd(&grad[MLP_OFF_W2 + k], g);
    }
    for (int u = t; u < H; u += blockDim.x) {
        float g = 0.0f;
        for (int s = 0; s < TB; s++) g += Z2[s][u];
        atomicAdd(&grad[MLP_OFF_B2 + u], g);
    }
    __syncthreads();
    // dZ1[s][v] = (sum_u dZ2[s][u] W2[u][v]) silu'(Z1[s][v])  (into Z1)
    for (int k = t; k < TB * H; k += blockDim.x) {
        const int s = k / H, v = k % H;
        float d = 0.0f;
        for (int u = 0; u < H; u++) d = fmaf(Z2[s][u], W2s[u][v], d);
        Z1[s][v] = d * dsilu(Z1[s][v]);
    }
    __syncthreads();
    // dW1[u][f] = sum_s dZ1[s][u] X[s][f]; db1[u] = sum_s dZ1[s][u]
    for (int k = t; k < H * I; k += blockDim.x) {
        const int u = k / I, f = k % I;
        float g = 0.0f;
        for (int s = 0; s < TB; s++) g = fmaf(Z1[s][u], X[s][f], g);
        atomicAdd(&grad[MLP_OFF_W1 + k], g);
    }
    for (int u = t; u < H; u += blockDim.x) {
        float g = 0.0f;
        for (int s = 0; s < TB; s++) g += Z1[s][u];
        atomicAdd(&grad[MLP_OFF_B1 + u], g);
    }
}

// AdamW on the FP32 master weights (decoupled weight decay on the matrices only)
__global__ void mlp_adamw_kernel(float* w, float* m, float* v, const float* g, int n, float lr, float b1, float b2,
                                 float eps, float wd, float bc1, float bc2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool matrix = (i >= MLP_OFF_W1 && i < MLP_OFF_B1) || (i >= MLP_OFF_W2 && i < MLP_OFF_B2) ||
                        (i >= MLP_OFF_W3 && i < MLP_OFF_B3);
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i];
    if (matrix) wi -= lr * wd * wi;
    wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
}

}  // namespace redgb

using namespace redgb;

struct rg_mlp {
    std::vector<float> w;  // FP32 master (host copy kept in sync on demand)
    float norm_mean[MLP_IN], norm_std[MLP_IN];
    float* d_w = nullptr;
    float* d_m = nullptr;
    float* d_v = nullptr;
    float* d_g = nullptr;
    __nv_bfloat16* d_wb = nullptr;
    float* d_loss = nullptr;
    int64_t step = 0;
    cudaStream_t st = nullptr;
};

namespace {

int sync_bf16(rg_mlp* m)
{
    mlp_to_bf16<<<(MLP_NPARAM + 255) / 256, 256, 0, m->st>>>(m->d_w, m->d_wb, MLP_NPARAM);
    RG_CUDA_CHECK(cudaGetLastError());
    return RG_OK;
}

template <class T>
int dalloc(T** p, size_t n)
{
    if (cudaMalloc((void**)p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return set_error(RG_ERR_NOMEM, "cudaMalloc (mlp)");
    }
    return RG_OK;
}

int create_impl(uint64_t seed, rg_mlp** out)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return set_error(RG_ERR_NO_DEVICE, "no CUDA device");
    }
    rg_mlp* m = new rg_mlp();
    m->w.assign(MLP_NPARAM, 0.0f);
    std::mt19937_64 rng(seed);
    auto init = [&](int off, int fan_out, int fan_in) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)(fan_in + fan_out)));
        for (int k = 0; k < fan_out * fan_in; k++) m->w[off + k] = nd(rng);
    };
    init(MLP_OFF_W1, MLP_HIDDEN, MLP_IN);
    init(MLP_OFF_W2, MLP_HIDDEN, MLP_HIDDEN);
    init(MLP_OFF_W3, 1, MLP_HIDDEN);
    for (int f = 0; f < MLP_IN; f++) {
        m->norm_mean[f] = 0.0f;
        m->norm_std[f] = 1.0f;
    }
    int rc = RG_OK;
    if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess) rc = set_error(RG_ERR_CUDA, "stream");
    if (!rc) rc = dalloc(&m->d_w, MLP_NPARAM);
    if (!rc) rc = dalloc(&m->d_m, MLP_NPARAM);
    if (!rc) rc = dalloc(&m->d_v, MLP_NPARAM);
    if (!rc) rc = dalloc(&m->d_g, MLP_NPARAM);
    if (!rc) rc = dalloc(&m->d_wb, MLP_NPARAM);
    if (!rc) rc = dalloc(&m->d_loss, 1);
    if (!rc && cudaMemcpy(m->d_w, m->w.data(), MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = set_error(RG_ERR_CUDA, "upload");
    if (!rc && cudaMemset(m->d_m, 0, MLP_NPARAM * sizeof(float)) != cudaSuccess) rc = RG_ERR_CUDA;
    if (!rc && cudaMemset(m->d_v, 0, MLP_NPARAM * sizeof(float)) != cudaSuccess) rc = RG_ERR_CUDA;
    if (!rc) rc = sync_bf16(m);
    if (!rc && cudaStreamSynchronize(m->st) != cudaSuccess) rc = set_error(RG_ERR_CUDA, "init");
    if (rc) {
        rg_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return RG_OK;
}

// standardised copy of the inputs
std::vector<float> standardise(const rg_mlp* m, const float* x, int n)
{
    std::vector<float> z((size_t)n * MLP_IN);
    for (int s = 0; s < n; s++)
        for (int f = 0; f < MLP_IN; f++)
            z[(size_t)s * MLP_IN + f] = (x[(size_t)s * MLP_IN + f] - m->norm_mean[f]) / m->norm_std[f];
    return z;
}

int run_tiles(rg_mlp* m, bool train, const float* d_x, const float* d_y, const int* d_idx, int n, float* d_out,
              float inv_batch)
{
    const int grid = (n + MLP_TB - 1) / MLP_TB;
    if (grid <= 0) return RG_OK;
    if (train)
        mlp_tile_kernel<true><<<grid, 256, 0, m->st>>>(m->d_wb, d_x, d_y, d_idx, n, inv_batch, d_out, m->d_g,
                                                       m->d_loss);
    else
        mlp_tile_kernel<false><<<grid, 256, 0, m->st>>>(m->d_wb, d_x, d_y, d_idx, n, inv_batch, d_out, nullptr,
                                                        nullptr);
    RG_CUDA_CHECK(cudaGetLastError());
    return RG_OK;
}

}  // namespace

extern "C" {

int rg_mlp_create(uint64_t seed, rg_mlp** out)
{
    if (!out) return set_error(RG_ERR_ARG, "null output");
    try {
        return create_impl(seed, out);
    } catch (const std::bad_alloc&) {
        return set_error(RG_ERR_NOMEM, "host allocation failed");
    }
}

int rg_mlp_destroy(rg_mlp* m)
{
    if (!m) return set_error(RG_ERR_ARG, "null network");
    if (m->st) cudaStreamSynchronize(m->st);
    cudaFree(m->d_w);
    cudaFree(m->d_m);
    cudaFree(m->d_v);
    cudaFree(m->d_g);
    cudaFree(m->d_wb);
    cudaFree(m->d_loss);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
    return RG_OK;
}

int rg_mlp_set_normalisation(rg_mlp* m, const float mean[MLP_IN], const float stdev[MLP_IN])
{
    if (!m || !mean || !stdev) return set_error(RG_ERR_ARG, "bad argument");
    for (int f = 0; f < MLP_IN; f++) {
        if (!(stdev[f] > 0.0f)) return set_error(RG_ERR_ARG, "standard deviation must be positive");
        m->norm_mean[f] = mean[f];
        m->norm_std[f] = stdev[f];
    }
    return RG_OK;
}

int rg_mlp_get_normalisation(rg_mlp* m, float mean[MLP_IN], float stdev[MLP_IN])
{
    if (!m || !mean || !stdev) return set_error(RG_ERR_ARG, "bad argument");
    for (int f = 0; f < MLP_IN; f++) {
        mean[f] = m->norm_mean[f];
        stdev[f] = m->norm_std[f];
    }
    return RG_OK;
}

int rg_mlp_get_params(rg_mlp* m, float* w, int n)
{
    if (!m || !w || n != MLP_NPARAM) return set_error(RG_ERR_ARG, "bad argument");
    RG_CUDA_CHECK(cudaMemcpy(w, m->d_w, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return RG_OK;
}

int rg_mlp_set_params(rg_mlp* m, const float* w, int n)
{
    if (!m || !w || n != MLP_NPARAM) return set_error(RG_ERR_ARG, "bad argument");
    RG_CUDA_CHECK(cudaMemcpy(m->d_w, w, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    int rc = sync_bf16(m);
    if (!rc) RG_CUDA_CHECK(cudaStreamSynchronize(m->st));
    return rc;
}

int rg_mlp_forward(rg_mlp* m, const float* x, int n, float* y)
{
    if (!m || n < 0 || (n > 0 && (!x || !y))) return set_error(RG_ERR_ARG, "bad argument");
    if (n == 0) return RG_OK;
    std::vector<float> z = standardise(m, x, n);
    float *d_x = nullptr, *d_o = nullptr;
    int rc = dalloc(&d_x, z.size());
    if (!rc) rc = dalloc(&d_o, (size_t)n);
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(d_x, z.data(), z.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
    if (!rc) rc = run_tiles(m, false, d_x, nullptr, nullptr, n, d_o, 0.0f);
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(y, d_o, n * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    if (!rc) RG_CUDA_CHECK(cudaStreamSynchronize(m->st));
    cudaFree(d_x);
    cudaFree(d_o);
    return rc;
}

// mean-squared-error gradient of one batch (no update): grads[MLP_NPARAM], loss
int rg_mlp_gradient(rg_mlp* m, const float* x, const float* y, int n, float* grads, float* loss)
{
    if (!m || n <= 0 || !x || !y || !grads) return set_error(RG_ERR_ARG, "bad argument");
    std::vector<float> z = standardise(m, x, n);
    float *d_x = nullptr, *d_y = nullptr;
    int rc = dalloc(&d_x, z.size());
    if (!rc) rc = dalloc(&d_y, (size_t)n);
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(d_x, z.data(), z.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(d_y, y, n * sizeof(float), cudaMemcpyHostToDevice, m->st));
    if (!rc) RG_CUDA_CHECK(cudaMemsetAsync(m->d_g, 0, MLP_NPARAM * sizeof(float), m->st));
    if (!rc) RG_CUDA_CHECK(cudaMemsetAsync(m->d_loss, 0, sizeof(float), m->st));
    if (!rc) rc = run_tiles(m, true, d_x, d_y, nullptr, n, nullptr, 1.0f / (float)n);
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(grads, m->d_g, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    float l = 0.0f;
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    if (!rc) RG_CUDA_CHECK(cudaStreamSynchronize(m->st));
    if (loss) *loss = l;
    cudaFree(d_x);
    cudaFree(d_y);
    return rc;
}

// AdamW training: `epochs` passes over the n samples in shuffled minibatches.
int rg_mlp_train(rg_mlp* m, const float* x, const float* y, int n, int epochs, int batch, float lr, float weight_decay,
                 uint64_t seed, float* final_loss)
{
    if (!m || !x || !y || n <= 0 || epochs <= 0 || batch <= 0 || !(lr > 0.0f))
        return set_error(RG_ERR_ARG, "bad argument");
    std::vector<float> z = standardise(m, x, n);
    float *d_x = nullptr, *d_y = nullptr;
    int* d_idx = nullptr;
    int rc = dalloc(&d_x, z.size());
    if (!rc) rc = dalloc(&d_y, (size_t)n);
    if (!rc) rc = dalloc(&d_idx, (size_t)n);
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(d_x, z.data(), z.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(d_y, y, n * sizeof(float), cudaMemcpyHostToDevice, m->st));
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    std::mt19937_64 rng(seed);
    float l = 0.0f;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs && !rc; ep++) {
        std::shuffle(idx.begin(), idx.end(), rng);
        RG_CUDA_CHECK(cudaMemcpyAsync(d_idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, m->st));
        for (int b0 = 0; b0 < n && !rc; b0 += batch) {
            const int nb = std::min(batch, n - b0);
            RG_CUDA_CHECK(cudaMemsetAsync(m->d_g, 0, MLP_NPARAM * sizeof(float), m->st));
            RG_CUDA_CHECK(cudaMemsetAsync(m->d_loss, 0, sizeof(float), m->st));
            rc = run_tiles(m, true, d_x, d_y, d_idx + b0, nb, nullptr, 1.0f / (float)nb);
            if (rc) break;
            m->step++;
            const float bc1 = 1.0f - std::pow(b1, (float)m->step), bc2 = 1.0f - std::pow(b2, (float)m->step);
            mlp_adamw_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, m->st>>>(m->d_w, m->d_m, m->d_v, m->d_g, MLP_NPARAM, lr,
                                                                        b1, b2, eps, weight_decay, bc1, bc2);
            RG_CUDA_CHECK(cudaGetLastError());
            rc = sync_bf16(m);
        }
    }
    if (!rc) RG_CUDA_CHECK(cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    if (!rc) RG_CUDA_CHECK(cudaStreamSynchronize(m->st));
    if (final_loss) *final_loss = l;
    cudaFree(d_x);
    cudaFree(d_y);
    cudaFree(d_idx);
    return rc;
}

}  // extern "C"

// access for the ensemble's proposer kernel
namespace redgb {
const void* mlp_device_weights(const rg_mlp* m) { return m ? (const void*)m->d_wb : nullptr; }
void mlp_normalisation(const rg_mlp* m, float* mean, float* stdev)
{
    for (int f = 0; f < MLP_IN; f++) {
        mean[f] = m->norm_mean[f];
        stdev[f] = m->norm_std[f];
    }
}
}  // namespace redgb
