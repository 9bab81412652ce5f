// btc_eval_sums_noalloc: the FP64 error sums of compute_metrics_gpu for
// callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code embedded in a
// host framework that owns every device allocation through its own pool (a
// caching allocator that has already reserved the memory, an engine that
// forbids allocation once it has started), and latency-critical loops that
// must not take the driver's allocation lock.  This entry point serves them:
// the caller passes device pointers for the inputs and for the three output
// sums, and the only scratch the reduction needs -- one partial triple per
// chunk of entries -- lives in a file-scope __device__ array that every GPU
// loading the library holds until the process exits.
//
// Limits and sharing:
//  * at most BTC_NOALLOC_MAX_ENTRIES entries per call (kChunk entries per
//    partial, kMaxPartials partials = 3 x 65536 doubles = 1.5 MiB of scratch);
//    larger n is rejected with BTC_ERR_RANGE before anything is launched;
//  * every call on a device shares the one array and overwrites the partials
//    it uses and the output, so nothing carries over from an earlier call,
//    but calls whose kernels overlap on the GPU (different streams, or
//    different host threads) race on the array and must be serialised by the
//    caller;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress while that device is current; make that first call
//    before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "btc_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 1024;          // entries reduced by one CTA into one partial
constexpr int kMaxPartials = 65536;   // scratch capacity in partials
constexpr int kGroup = 8;             // lanes per entry
constexpr int kMaxDevices = 64;
static_assert((long long)kChunk * kMaxPartials == BTC_NOALLOC_MAX_ENTRIES, "limit mismatch");

static __device__ __align__(256) double g_noalloc_partials[3 * kMaxPartials];

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

// Variant of k_metrics (kernels.cu): fixed chunks instead of a grid-stride
// loop, so the partials (and the final fixed-order sum) do not depend on the
// device's SM count; rows of any stride, read element by element.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_sums_chunked(const int32_t* xyz, const double* val, long long n,
                                                          const T* A, const T* B, const T* C, int R,
                                                          long long stride, double* partials)
{
    const int lane = threadIdx.x & 31;
    const int sub = lane / kGroup, gl = lane % kGroup;
    const int warp = threadIdx.x >> 5;
    constexpr int EPW = 32 / kGroup;
    constexpr int WARPS = kThreads / 32;
    const long long begin = (long long)blockIdx.x * kChunk;
    const long long end = begin + kChunk < n ? begin + kChunk : n;
    double sse = 0, sae = 0, r2 = 0;
    for (long long ib = begin + warp * EPW; ib < end; ib += WARPS * EPW) {
        const long long i = ib + sub;
        const bool act = i < end;
        T p = T(0);
        if (act) {
            const T* a = A + (long long)xyz[3 * i] * stride;
            const T* b = B + (long long)xyz[3 * i + 1] * stride;
            const T* c = C + (long long)xyz[3 * i + 2] * stride;
            for (int q = gl; q < R; q += kGroup)
                p = fma(a[q], b[q] * c[q], p);
        }
#pragma unroll
        for (int o = kGroup / 2; o > 0; o >>= 1)
            p += __shfl_xor_sync(0xffffffffu, p, o);
        if (act && gl == 0) {
            const double ref = val[i];
            const double err = ref - (double)p;
            sae += fabs(err);
            sse += err * err;
            r2 += ref * ref;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sse += __shfl_xor_sync(0xffffffffu, sse, o);
        sae += __shfl_xor_sync(0xffffffffu, sae, o);
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    }
    __shared__ double red[3][WARPS];
    if (lane == 0) {
        red[0][warp] = sse;
        red[1][warp] = sae;
        red[2][warp] = r2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0;
        for (int k = 0; k < WARPS; k++)
            s += red[threadIdx.x][k];
        partials[3 * (long long)blockIdx.x + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) k_sums_final(const double* partials, int nblk, double* out)
{
    __shared__ double red[3][256];
    double s[3] = {0, 0, 0};
    for (int b = threadIdx.x; b < nblk; b += 256)
        for (int k = 0; k < 3; k++)
            s[k] += partials[3 * (long long)b + k];
    for (int k = 0; k < 3; k++)
        red[k][threadIdx.x] = s[k];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int k = 0; k < 3; k++)
                red[k][threadIdx.x] += red[k][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 3)
        out[threadIdx.x] = red[threadIdx.x][0];
}

// Device address of the scratch array for the current device, looked up
// once per device.
btc_status scratch_for_current_device(double** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return BTC_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices)
        return BTC_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p)
            return BTC_ERR_CUDA;
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
    return BTC_OK;
}

}  // namespace

extern "C" btc_status btc_eval_sums_noalloc(const int32_t* xyz, const double* val, int64_t n, const void* A,
                                           const void* B, const void* C, int32_t dtype, int32_t rank,
                                           int64_t row_stride, double* sums, void* stream)
{
    if (!sums || n < 0 || rank <= 0 || rank > 128 || row_stride < rank)
        return BTC_ERR_ARG;
    if (dtype != BTC_DTYPE_F32 && dtype != BTC_DTYPE_F64)
        return BTC_ERR_UNSUPPORTED;
    if (n > BTC_NOALLOC_MAX_ENTRIES)
        return BTC_ERR_RANGE;
    if (n > 0 && (!xyz || !val || !A || !B || !C))
        return BTC_ERR_ARG;
    double* scratch = nullptr;
    btc_status rc = scratch_for_current_device(&scratch);
    if (rc != BTC_OK)
        return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nblk = (int)((n + kChunk - 1) / kChunk);
    if (nblk > 0) {
        if (dtype == BTC_DTYPE_F64)
            k_sums_chunked<double><<<nblk, kThreads, 0, st>>>(xyz, val, n, (const double*)A, (const double*)B,
                                                              (const double*)C, rank, row_stride, scratch);
        else
            k_sums_chunked<float><<<nblk, kThreads, 0, st>>>(xyz, val, n, (const float*)A, (const float*)B,
                                                             (const float*)C, rank, row_stride, scratch);
        if (cudaGetLastError() != cudaSuccess)
            return BTC_ERR_CUDA;
    }
    k_sums_final<<<1, 256, 0, st>>>(scratch, nblk, sums);
    if (cudaGetLastError() != cudaSuccess)
        return BTC_ERR_CUDA;
    return BTC_OK;
}
