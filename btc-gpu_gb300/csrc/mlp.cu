// The learned cost model: a small MLP (nin -> nh -> nh -> 1, tanh hidden
// units) trained and evaluated with this file's own CUDA kernels.
//
//   k_mlp_forward   one thread per sample; the weights sit in shared memory
//   k_mlp_grad      one warp per 32 samples: each lane runs its sample forward
//                   and backward in registers, every weight's gradient is
//                   reduced across the warp with xor-shuffles and added once per
//                   warp to a shared-memory accumulator, then once per CTA to
//                   global memory; the loss is the mean squared error
//   k_mlp_adam      Adam update (Kingma & Ba, 2015), one thread per weight
//
// Weight layout (flat, float): W1[nh][nin], b1[nh], W2[nh][nh], b2[nh],
// w3[nh], b3.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "btc_gpu.h"

namespace {

constexpr int kMaxIn = 16;
constexpr int kH = 32;  // hidden width the kernels are written for

struct Layout {
    int nin, nh, w1, b1, w2, b2, w3, b3, total;
    Layout(int in, int h) : nin(in), nh(h)
    {
        w1 = 0;
        b1 = w1 + h * in;
        w2 = b1 + h;
        b2 = w2 + h * h;
        w3 = b2 + h;
        b3 = w3 + h;
        total = b3 + 1;
    }
};

__device__ __forceinline__ float mlp_fwd(const float* P, const float* x, int nin, float* h1, float* h2)
{
    const float* W1 = P;
    const float* B1 = W1 + kH * nin;
    const float* W2 = B1 + kH;
    const float* B2 = W2 + kH * kH;
    const float* W3 = B2 + kH;
    const float B3 = W3[kH];
#pragma unroll 4
    for (int i = 0; i < kH; i++) {
        float z = B1[i];
        for (int k = 0; k < nin; k++)
            z = fmaf(W1[i * nin + k], x[k], z);
        h1[i] = tanhf(z);
    }
    for (int i = 0; i < kH; i++) {
        float z = B2[i];
#pragma unroll
        for (int k = 0; k < kH; k++)
            z = fmaf(W2[i * kH + k], h1[k], z);
        h2[i] = tanhf(z);
    }
    float y = B3;
#pragma unroll
    for (int i = 0; i < kH; i++)
        y = fmaf(W3[i], h2[i], y);
    return y;
}

__global__ void __launch_bounds__(256) k_mlp_forward(const float* __restrict__ params, int nparam, int nin,
                                                     const float* __restrict__ x, long long n, float* __restrict__ y)
{
    extern __shared__ float sp[];
    for (int i = threadIdx.x; i < nparam; i += blockDim.x)
        sp[i] = params[i];
    __syncthreads();
    float h1[kH], h2[kH], xi[kMaxIn];
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += (long long)gridDim.x * blockDim.x) {
        for (int k = 0; k < nin; k++)
            xi[k] = x[s * nin + k];
        y[s] = mlp_fwd(sp, xi, nin, h1, h2);
    }
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// adds the warp's sum of v to acc[p]; lane p % 32 does the add
__device__ __forceinline__ void warp_add(float* acc, int p, float v, int lane)
{
    v = warp_sum(v);
    if (lane == (p & 31))
        atomicAdd(&acc[p], v);
}

__global__ void __launch_bounds__(256) k_mlp_grad(const float* __restrict__ params, int nparam, int nin,
                                                  const float* __restrict__ x, const float* __restrict__ t,
                                                  long long n, float inv_n, float* __restrict__ grad,
                                                  float* __restrict__ loss)
{
    extern __shared__ float sm[];
    float* sp = sm;
    float* sg = sm + nparam;
    for (int i = threadIdx.x; i < nparam; i += blockDim.x) {
        sp[i] = params[i];
        sg[i] = 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const float* W2 = sp + kH * nin + kH;
    const float* W3 = W2 + kH * kH + kH;
    const int o_b1 = kH * nin, o_w2 = o_b1 + kH, o_b2 = o_w2 + kH * kH, o_w3 = o_b2 + kH, o_b3 = o_w3 + kH;
    float lsum = 0.f;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long base = warp * 32; base < n; base += nwarps * 32) {
        const long long s = base + lane;
        const bool act = s < n;
        float xi[kMaxIn], h1[kH], h2[kH];
        for (int k = 0; k < nin; k++)
            xi[k] = act ? x[s * nin + k] : 0.f;
        const float y = mlp_fwd(sp, xi, nin, h1, h2);
        const float e = act ? (y - t[s]) : 0.f;
        lsum += e * e;
        const float dy = 2.f * e * inv_n;  // d(mean sq. error)/dy
        // output layer
        warp_add(sg, o_b3, dy, lane);
        float dz2[kH];
#pragma unroll
        for (int i = 0; i < kH; i++) {
            warp_add(sg, o_w3 + i, dy * h2[i], lane);
            dz2[i] = dy * W3[i] * (1.f - h2[i] * h2[i]);
        }
        // second hidden layer
        float dh1[kH];
#pragma unroll
        for (int k = 0; k < kH; k++)
            dh1[k] = 0.f;
        for (int i = 0; i < kH; i++) {
            warp_add(sg, o_b2 + i, dz2[i], lane);
#pragma unroll
            for (int k = 0; k < kH; k++) {
                warp_add(sg, o_w2 + i * kH + k, dz2[i] * h1[k], lane);
                dh1[k] = fmaf(W2[i * kH + k], dz2[i], dh1[k]);
            }
        }
        // first hidden layer
        for (int i = 0; i < kH; i++) {
            const float dz1 = dh1[i] * (1.f - h1[i] * h1[i]);
            warp_add(sg, o_b1 + i, dz1, lane);
            for (int k = 0; k < nin; k++)
                warp_add(sg, i * nin + k, dz1 * xi[k], lane);
        }
    }
    lsum = warp_sum(lsum);
    if (lane == 0)
        atomicAdd(loss, lsum * inv_n);
    __syncthreads();
    for (int i = threadIdx.x; i < nparam; i += blockDim.x)
        atomicAdd(&grad[i], sg[i]);
}

__global__ void k_mlp_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2,
                           float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

struct btc_mlp {
    Layout L{1, kH};
    int device = 0;
    cudaStream_t stream = nullptr;
    float* p = nullptr;
    float* g = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* loss = nullptr;
    long long adam_t = 0;
};

namespace {

btc_status cuda_ok(cudaError_t e) { return e == cudaSuccess ? BTC_OK : BTC_ERR_CUDA; }

#define MCK(call)                                        \
    do {                                                 \
        if ((call) != cudaSuccess)                       \
            return BTC_ERR_CUDA;                         \
    } while (0)

int grid_for(long long n, int per)
{
    long long b = (n + per - 1) / per;
    return (int)std::max<long long>(1, std::min<long long>(b, 1024));
}

btc_status upload_xy(const float* x, const float* y, long long n, int nin, float** dx, float** dy)
{
    MCK(cudaMalloc((void**)dx, std::max<size_t>(16, (size_t)n * nin * 4)));
    if (n > 0)
        MCK(cudaMemcpy(*dx, x, (size_t)n * nin * 4, cudaMemcpyHostToDevice));
    if (dy) {
        MCK(cudaMalloc((void**)dy, std::max<size_t>(16, (size_t)n * 4)));
        if (n > 0)
            MCK(cudaMemcpy(*dy, y, (size_t)n * 4, cudaMemcpyHostToDevice));
    }
    return BTC_OK;
}

btc_status grad_on_device(btc_mlp* m, const float* dx, const float* dy, long long n)
{
    const int P = m->L.total;
    MCK(cudaMemsetAsync(m->g, 0, (size_t)P * 4, m->stream));
    MCK(cudaMemsetAsync(m->loss, 0, 4, m->stream));
    if (n == 0)
        return BTC_OK;
    const size_t smem = (size_t)2 * P * 4;
    k_mlp_grad<<<grid_for(n, 256), 256, smem, m->stream>>>(m->p, P, m->L.nin, dx, dy, n, 1.f / (float)n, m->g,
                                                           m->loss);
    return cuda_ok(cudaGetLastError());
}

}  // namespace

extern "C" {

btc_status btc_mlp_create(int32_t n_in, int32_t n_hidden, uint64_t seed, int32_t device, btc_mlp** out)
{
    if (!out || n_in <= 0 || n_in > kMaxIn || n_hidden != kH)
        return BTC_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess)
        return BTC_ERR_CUDA;
    btc_mlp* m = new (std::nothrow) btc_mlp();
    if (!m)
        return BTC_ERR_ALLOC;
    m->L = Layout(n_in, n_hidden);
    m->device = device;
    const int P = m->L.total;
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void**)&m->p, P * 4) != cudaSuccess || cudaMalloc((void**)&m->g, P * 4) != cudaSuccess ||
        cudaMalloc((void**)&m->m, P * 4) != cudaSuccess || cudaMalloc((void**)&m->v, P * 4) != cudaSuccess ||
        cudaMalloc((void**)&m->loss, 16) != cudaSuccess) {
        btc_mlp_destroy(m);
        return BTC_ERR_CUDA;
    }
    // Glorot-uniform weights from a seeded generator, zero biases
    std::vector<float> h((size_t)P, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fan_in, int fan_out, int count) {
        std::uniform_real_distribution<float> d(-std::sqrt(6.f / (fan_in + fan_out)),
                                                std::sqrt(6.f / (fan_in + fan_out)));
        for (int i = 0; i < count; i++)
            h[(size_t)off + i] = d(rng);
    };
    fill(m->L.w1, n_in, kH, kH * n_in);
    fill(m->L.w2, kH, kH, kH * kH);
    fill(m->L.w3, kH, 1, kH);
    if (cudaMemcpy(m->p, h.data(), (size_t)P * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->m, 0, (size_t)P * 4) != cudaSuccess || cudaMemset(m->v, 0, (size_t)P * 4) != cudaSuccess) {
        btc_mlp_destroy(m);
        return BTC_ERR_CUDA;
    }
    *out = m;
    return BTC_OK;
}

btc_status btc_mlp_destroy(btc_mlp* m)
{
    if (!m)
        return BTC_OK;
    cudaSetDevice(m->device);
    if (m->stream)
        cudaStreamSynchronize(m->stream);
    cudaFree(m->p);
    cudaFree(m->g);
    cudaFree(m->m);
    cudaFree(m->v);
    cudaFree(m->loss);
    if (m->stream)
        cudaStreamDestroy(m->stream);
    delete m;
    return BTC_OK;
}

btc_status btc_mlp_param_count(const btc_mlp* m, int64_t* n)
{
    if (!m || !n)
        return BTC_ERR_ARG;
    *n = m->L.total;
    return BTC_OK;
}

btc_status btc_mlp_get_params(btc_mlp* m, float* host)
{
    if (!m || !host)
        return BTC_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    MCK(cudaMemcpy(host, m->p, (size_t)m->L.total * 4, cudaMemcpyDeviceToHost));
    return BTC_OK;
}

btc_status btc_mlp_set_params(btc_mlp* m, const float* host)
{
    if (!m || !host)
        return BTC_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    MCK(cudaMemcpy(m->p, host, (size_t)m->L.total * 4, cudaMemcpyHostToDevice));
    MCK(cudaMemset(m->m, 0, (size_t)m->L.total * 4));
    MCK(cudaMemset(m->v, 0, (size_t)m->L.total * 4));
    m->adam_t = 0;
    return BTC_OK;
}

btc_status btc_mlp_gradient(btc_mlp* m, const float* x, const float* y, int64_t n, float* grad, double* loss)
{
    if (!m || n < 0 || (n > 0 && (!x || !y)) || !grad)
        return BTC_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    float *dx = nullptr, *dy = nullptr;
    btc_status rc = upload_xy(x, y, n, m->L.nin, &dx, &dy);
    if (rc == BTC_OK)
        rc = grad_on_device(m, dx, dy, n);
    float l = 0;
    if (rc == BTC_OK && (cudaMemcpyAsync(grad, m->g, (size_t)m->L.total * 4, cudaMemcpyDeviceToHost, m->stream) !=
                             cudaSuccess ||
                         cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
                         cudaStreamSynchronize(m->stream) != cudaSuccess))
        rc = BTC_ERR_CUDA;
    if (loss)
        *loss = l;
    cudaFree(dx);
    cudaFree(dy);
    return rc;
}

btc_status btc_mlp_train(btc_mlp* m, const float* x, const float* y, int64_t n, int32_t steps, float lr,
                         double* final_loss)
{
    if (!m || n <= 0 || !x || !y || steps < 0 || !(lr > 0))
        return BTC_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    float *dx = nullptr, *dy = nullptr;
    btc_status rc = upload_xy(x, y, n, m->L.nin, &dx, &dy);
    const int P = m->L.total;
    for (int s = 0; s < steps && rc == BTC_OK; s++) {
        rc = grad_on_device(m, dx, dy, n);
        if (rc != BTC_OK)
            break;
        m->adam_t++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)m->adam_t), c2 = 1.f - std::pow(b2, (float)m->adam_t);
        k_mlp_adam<<<(P + 255) / 256, 256, 0, m->stream>>>(m->p, m->g, m->m, m->v, P, lr, b1, b2, 1e-8f, c1, c2);
        rc = cuda_ok(cudaGetLastError());
    }
    if (rc == BTC_OK)
        rc = grad_on_device(m, dx, dy, n);  // loss at the final weights
    float l = 0;
    if (rc == BTC_OK && (cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
                         cudaStreamSynchronize(m->stream) != cudaSuccess))
        rc = BTC_ERR_CUDA;
    if (final_loss)
        *final_loss = l;
    cudaFree(dx);
    cudaFree(dy);
    return rc;
}

int32_t btc_mlp_inputs(const btc_mlp* m) { return m ? (int32_t)m->L.nin : 0; }

btc_status btc_mlp_predict(btc_mlp* m, const float* x, int64_t n, float* y)
{
    if (!m || n < 0 || (n > 0 && (!x || !y)))
        return BTC_ERR_ARG;
    if (n == 0)
        return BTC_OK;
    MCK(cudaSetDevice(m->device));
    float *dx = nullptr, *dy = nullptr;
    btc_status rc = upload_xy(x, nullptr, n, m->L.nin, &dx, nullptr);
    if (rc == BTC_OK && cudaMalloc((void**)&dy, (size_t)n * 4) != cudaSuccess)
        rc = BTC_ERR_CUDA;
    if (rc == BTC_OK) {
        k_mlp_forward<<<grid_for(n, 256), 256, (size_t)m->L.total * 4, m->stream>>>(m->p, m->L.total, m->L.nin,
                                                                                   dx, n, dy);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(y, dy, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
            cudaStreamSynchronize(m->stream) != cudaSuccess)
            rc = BTC_ERR_CUDA;
    }
    cudaFree(dx);
    cudaFree(dy);
    return rc;
}

}  // extern "C"
