// sm_103a kernels of the CP-SGD path.
//
// The path is a sparse gather/scatter with about one flop per byte: it is
// bound by memory traffic (HBM for the entry stream, L2 for factor rows that
// stay resident), not by tensor cores.  Every kernel therefore works on
// 16-byte vectors: one entry is one int4 (x, y, z, value) and one factor-row
// slice is one float4 / double2 per lane.
//
//  k_hogwild   -- the reference GPUs kernel's update (sgd_Kernel.cu:313-398)
//                 spread over every SM: work items (a chunk of one slot) are
//                 swept in schedule order by all warps; a group of G lanes
//                 owns one entry, gathers its three rows from L2 (ld.cg, so a
//                 hot row is never served stale from L1), reduces the dot with
//                 xor-shuffles and adds the three row deltas with vector
//                 atomics (red.global.add.v4.f32 / f64).
//  k_det       -- deterministic replay: one warp per slot, entries in block
//                 order, every product rounded exactly as written, so the
//                 FP64 instance equals the serial FP64 rule bit for bit.
//  k_metrics   -- compute_metrics_gpu (sgd_Kernel.cu:64-120) with FP64 sums,
//                 per-CTA partials and a fixed-order final sum.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace btc {
namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T>
struct VT;
template <>
struct VT<float> {
    static constexpr int N = 4;
};
template <>
struct VT<double> {
    static constexpr int N = 2;
};

__device__ __forceinline__ void ldrow(const float* p, float* r)
{
    float4 v = __ldcg(reinterpret_cast<const float4*>(p));
    r[0] = v.x;
    r[1] = v.y;
    r[2] = v.z;
    r[3] = v.w;
}
__device__ __forceinline__ void ldrow(const double* p, double* r)
{
    double2 v = __ldcg(reinterpret_cast<const double2*>(p));
    r[0] = v.x;
    r[1] = v.y;
}
__device__ __forceinline__ void ldrow_ro(const float* p, float* r)
{
    float4 v = __ldg(reinterpret_cast<const float4*>(p));
    r[0] = v.x;
    r[1] = v.y;
    r[2] = v.z;
    r[3] = v.w;
}
__device__ __forceinline__ void ldrow_ro(const double* p, double* r)
{
    double2 v = __ldg(reinterpret_cast<const double2*>(p));
    r[0] = v.x;
    r[1] = v.y;
}
__device__ __forceinline__ void ldrow_ro(const unsigned short* p, float* r)
{
    uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
    r[0] = __uint_as_float(v.x << 16);
    r[1] = __uint_as_float(v.x & 0xffff0000u);
    r[2] = __uint_as_float(v.y << 16);
    r[3] = __uint_as_float(v.y & 0xffff0000u);
}
// a vector add that returns nothing (red, not atom): no register waits on
// the old value
__device__ __forceinline__ void addrow(float* p, const float* d)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(d[0]), "f"(d[1]), "f"(d[2]),
                 "f"(d[3])
                 : "memory");
}
__device__ __forceinline__ void addrow(double* p, const double* d)
{
    atomicAdd(p, d[0]);
    atomicAdd(p + 1, d[1]);
}

template <typename T>
__device__ __forceinline__ T entry_value(const int4& e, const double* val64, long long idx);
template <>
__device__ __forceinline__ float entry_value<float>(const int4& e, const double*, long long)
{
    return __int_as_float(e.w);
}
template <>
__device__ __forceinline__ double entry_value<double>(const int4&, const double* val64, long long idx)
{
    return __ldg(val64 + idx);
}

template <typename T, int G, int NV>
__global__ void __launch_bounds__(256) k_hogwild(SgdArgs a)
{
    constexpr int VN = VT<T>::N;
    constexpr int EPW = 32 / G;
    constexpr int E = NV * VN;
    const int lane = threadIdx.x & 31;
    const int sub = lane / G;
    const int gl = lane % G;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const T* coe = static_cast<const T*>(a.slot_coe);
    T* A = static_cast<T*>(a.A);
    T* B = static_cast<T*>(a.B);
    T* C = static_cast<T*>(a.C);
    const T reg = (T)a.reg;
    const int Rp = a.Rp;

    for (long long it = warp; it < a.nitems; it += nwarps) {
        const int2 item = __ldg(&a.items[it]);
        const long long base = __ldg(&a.slot_off[item.x]) + item.y;
        const int cnt = min(a.chunk, __ldg(&a.slot_nnz[item.x]) - item.y);
        const T cx = __ldg(&coe[3 * item.x]);
        const T cy = __ldg(&coe[3 * item.x + 1]);
        const T cz = __ldg(&coe[3 * item.x + 2]);
        for (int e0 = 0; e0 < cnt; e0 += 32) {
            const int nh = min(32, cnt - e0);
            int4 my = make_int4(0, 0, 0, 0);
            if (lane < nh)
                my = __ldcs(&a.coo[base + e0 + lane]);
            for (int k = 0; k < nh; k += EPW) {
                const int src = k + sub;
                int4 en;
                en.x = __shfl_sync(FULL, my.x, src);
                en.y = __shfl_sync(FULL, my.y, src);
                en.z = __shfl_sync(FULL, my.z, src);
                en.w = __shfl_sync(FULL, my.w, src);
                const bool act = src < nh;
                T ra[E], rb[E], rc[E];
                T p = T(0);
                T v = T(0);
                if (act) {
                    v = entry_value<T>(en, a.val64, base + e0 + src);
                    const T* pa = A + (size_t)en.x * Rp + gl * VN;
                    const T* pb = B + (size_t)en.y * Rp + gl * VN;
                    const T* pc = C + (size_t)en.z * Rp + gl * VN;
#pragma unroll
                    for (int j = 0; j < NV; j++) {
                        ldrow(pa + j * G * VN, ra + j * VN);
                        ldrow(pb + j * G * VN, rb + j * VN);
                        ldrow(pc + j * G * VN, rc + j * VN);
                    }
#pragma unroll
                    for (int i = 0; i < E; i++)
                        p = fma(ra[i], rb[i] * rc[i], p);
                }
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1)
                    p += __shfl_xor_sync(FULL, p, o);
                if (act) {
                    const T err = v - p;
                    T da[E], db[E], dc[E];
#pragma unroll
                    for (int i = 0; i < E; i++) {
                        da[i] = cx * (err * (rb[i] * rc[i]) - reg * ra[i]);
                        db[i] = cy * (err * (ra[i] * rc[i]) - reg * rb[i]);
                        dc[i] = cz * (err * (ra[i] * rb[i]) - reg * rc[i]);
                    }
                    T* qa = A + (size_t)en.x * Rp + gl * VN;
                    T* qb = B + (size_t)en.y * Rp + gl * VN;
                    T* qc = C + (size_t)en.z * Rp + gl * VN;
#pragma unroll
                    for (int j = 0; j < NV; j++) {
                        addrow(qa + j * G * VN, da + j * VN);
                        addrow(qb + j * G * VN, db + j * VN);
                        addrow(qc + j * G * VN, dc + j * VN);
                    }
                }
            }
        }
    }
}

// exactly rounded helpers for the deterministic replay
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T>
__global__ void __launch_bounds__(128) k_det(const int* wave_slots, int n, SgdArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (w >= n)
        return;  // the whole warp leaves together
    T* sa = reinterpret_cast<T*>(smem_raw) + (size_t)(threadIdx.x >> 5) * 3 * a.Rp;
    T* sb = sa + a.Rp;
    T* sc = sb + a.Rp;
    const int s = wave_slots[w];
    const long long off = a.slot_off[s];
    const int nnz = a.slot_nnz[s];
    const T* coe = static_cast<const T*>(a.slot_coe);
    const T cx = coe[3 * s], cy = coe[3 * s + 1], cz = coe[3 * s + 2];
    const T reg = (T)a.reg;
    T* A = static_cast<T*>(a.A);
    T* B = static_cast<T*>(a.B);
    T* C = static_cast<T*>(a.C);
    const int R = a.R, Rp = a.Rp;
    for (int t = 0; t < nnz; t++) {
        const int4 e = __ldg(&a.coo[off + t]);
        const T v = entry_value<T>(e, a.val64, off + t);
        T* pa = A + (size_t)e.x * Rp;
        T* pb = B + (size_t)e.y * Rp;
        T* pc = C + (size_t)e.z * Rp;
        for (int q = lane; q < R; q += 32) {
            sa[q] = __ldcg(pa + q);
            sb[q] = __ldcg(pb + q);
            sc[q] = __ldcg(pc + q);
        }
        __syncwarp();
        T dot = T(0);
        for (int q = 0; q < R; q++)
            dot = fma_rn(sa[q], mul_rn(sb[q], sc[q]), dot);
        const T err = sub_rn(v, dot);
        for (int q = lane; q < R; q += 32) {
            const T av = sa[q], bv = sb[q], cv = sc[q];
            const T na = add_rn(av, mul_rn(cx, sub_rn(mul_rn(err, mul_rn(bv, cv)), mul_rn(reg, av))));
            const T nb = add_rn(bv, mul_rn(cy, sub_rn(mul_rn(err, mul_rn(av, cv)), mul_rn(reg, bv))));
            const T nc = add_rn(cv, mul_rn(cz, sub_rn(mul_rn(err, mul_rn(av, bv)), mul_rn(reg, cv))));
            __stcg(pa + q, na);
            __stcg(pb + q, nb);
            __stcg(pc + q, nc);
        }
        __syncwarp();
    }
}

// The lock-free rule (sgd_Kernel.cu:401-451) on one warp per block: entries
// in block order; per element the A row moves first, B from the new A, C
// from the new A and B.  Products are rounded as written: dot as
// fma(a * b, c, dot), each update x + lr * ((e * u) * v - reg * x).
template <typename T>
__global__ void __launch_bounds__(128) k_lf(const int* wave_slots, int n, SgdArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (w >= n)
        return;  // the whole warp leaves together
    T* sa = reinterpret_cast<T*>(smem_raw) + (size_t)(threadIdx.x >> 5) * 3 * a.Rp;
    T* sb = sa + a.Rp;
    T* sc = sb + a.Rp;
    const int s = wave_slots[w];
    const long long off = a.slot_off[s];
    const int nnz = a.slot_nnz[s];
    const T lr = static_cast<const T*>(a.slot_coe)[3 * s];  // coe 1 times lr
    const T reg = (T)a.reg;
    T* A = static_cast<T*>(a.A);
    T* B = static_cast<T*>(a.B);
    T* C = static_cast<T*>(a.C);
    const int R = a.R, Rp = a.Rp;
    for (int t = 0; t < nnz; t++) {
        const int4 e = __ldg(&a.coo[off + t]);
        const T v = entry_value<T>(e, a.val64, off + t);
        T* pa = A + (size_t)e.x * Rp;
        T* pb = B + (size_t)e.y * Rp;
        T* pc = C + (size_t)e.z * Rp;
        for (int q = lane; q < R; q += 32) {
            sa[q] = __ldcg(pa + q);
            sb[q] = __ldcg(pb + q);
            sc[q] = __ldcg(pc + q);
        }
        __syncwarp();
        T dot = T(0);
        for (int q = 0; q < R; q++)
            dot = fma_rn(mul_rn(sa[q], sb[q]), sc[q], dot);
        const T err = sub_rn(v, dot);
        for (int q = lane; q < R; q += 32) {
            const T av = sa[q], bv = sb[q], cv = sc[q];
            const T na = add_rn(av, mul_rn(lr, sub_rn(mul_rn(mul_rn(err, bv), cv), mul_rn(reg, av))));
            const T nb = add_rn(bv, mul_rn(lr, sub_rn(mul_rn(mul_rn(err, na), cv), mul_rn(reg, bv))));
            const T nc = add_rn(cv, mul_rn(lr, sub_rn(mul_rn(mul_rn(err, nb), na), mul_rn(reg, cv))));
            __stcg(pa + q, na);
            __stcg(pb + q, nb);
            __stcg(pc + q, nc);
        }
        __syncwarp();
    }
}

template <typename T, int G, int NV, typename ST = T>
__global__ void __launch_bounds__(kMetricThreads) k_metrics(const int4* coo, const double* val,
                                                           long long n, const ST* A, const ST* B,
                                                           const ST* C, int Rp, double* partials)
{
    constexpr int VN = VT<T>::N;
    constexpr int EPW = 32 / G;
    constexpr int E = NV * VN;
    const int lane = threadIdx.x & 31;
    const int sub = lane / G;
    const int gl = lane % G;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    double sse = 0, sae = 0, r2 = 0;
    for (long long ib = warp * EPW; ib < n; ib += nwarps * EPW) {
        const long long i = ib + sub;
        const bool act = i < n;
        T p = T(0);
        if (act) {
            const int4 e = __ldcs(&coo[i]);
            T ra[E], rb[E], rc[E];
#pragma unroll
            for (int j = 0; j < NV; j++) {
                ldrow_ro(A + (size_t)e.x * Rp + (j * G + gl) * VN, ra + j * VN);
                ldrow_ro(B + (size_t)e.y * Rp + (j * G + gl) * VN, rb + j * VN);
                ldrow_ro(C + (size_t)e.z * Rp + (j * G + gl) * VN, rc + j * VN);
            }
#pragma unroll
            for (int k = 0; k < E; k++)
                p = fma(ra[k], rb[k] * rc[k], p);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
            p += __shfl_xor_sync(FULL, p, o);
        if (act && gl == 0) {
            const double ref = __ldcs(&val[i]);
            const double err = ref - (double)p;
            sae += fabs(err);
            sse += err * err;
            r2 += ref * ref;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sse += __shfl_xor_sync(FULL, sse, o);
        sae += __shfl_xor_sync(FULL, sae, o);
        r2 += __shfl_xor_sync(FULL, r2, o);
    }
    __shared__ double red[3][kMetricThreads / 32];
    const int wid = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][wid] = sse;
        red[1][wid] = sae;
        red[2][wid] = r2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0;
        for (int k = 0; k < kMetricThreads / 32; k++)
            s += red[threadIdx.x][k];
        partials[3 * (size_t)blockIdx.x + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) k_metrics_final(const double* partials, int nblk, double* result)
{
    __shared__ double red[3][256];
    double s[3] = {0, 0, 0};
    for (int b = threadIdx.x; b < nblk; b += 256)
        for (int k = 0; k < 3; k++)
            s[k] += partials[3 * (size_t)b + k];
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
        result[threadIdx.x] = red[threadIdx.x][0];
}

// (G, NV) for a rank: G lanes per entry, NV 16-byte vectors per lane per row
template <typename T>
void pick_shape(int R, int& G, int& NV)
{
    constexpr int VN = VT<T>::N;
    NV = 1;
    G = 1;
    while (G * VN < R && G < 32)
        G *= 2;
    while (G * VN * NV < R)
        NV++;
}

template <typename T>
cudaError_t hogwild_t(const SgdArgs& a, int grid, int block, cudaStream_t st)
{
    int G, NV;
    pick_shape<T>(a.R, G, NV);
#define BTC_HW(g, nv)                                             \
    if (G == g && NV == nv) {                                     \
        k_hogwild<T, g, nv><<<grid, block, 0, st>>>(a);           \
        return cudaGetLastError();                                \
    }
    BTC_HW(1, 1) BTC_HW(2, 1) BTC_HW(4, 1) BTC_HW(8, 1) BTC_HW(16, 1) BTC_HW(32, 1)
    BTC_HW(32, 2)
#undef BTC_HW
    return cudaErrorInvalidValue;
}

template <typename T>
int hogwild_occ(int R, int block)
{
    int G, NV, n = 0;
    pick_shape<T>(R, G, NV);
#define BTC_OC(g, nv)                                                                          \
    if (G == g && NV == nv) {                                                                  \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_hogwild<T, g, nv>, block, 0);      \
        return n;                                                                              \
    }
    BTC_OC(1, 1) BTC_OC(2, 1) BTC_OC(4, 1) BTC_OC(8, 1) BTC_OC(16, 1) BTC_OC(32, 1)
    BTC_OC(32, 2)
#undef BTC_OC
    return 1;
}

template <typename T, typename ST = T>
cudaError_t metrics_t(const int4* coo, const double* val, long long n, const ST* A, const ST* B,
                      const ST* C, int R, int Rp, double* partials, int grid, double* result,
                      cudaStream_t st)
{
    int G, NV;
    pick_shape<T>(R, G, NV);
#define BTC_MT(g, nv)                                                                              \
    if (G == g && NV == nv) {                                                                      \
        k_metrics<T, g, nv, ST><<<grid, kMetricThreads, 0, st>>>(coo, val, n, A, B, C, Rp, partials); \
        cudaError_t e = cudaGetLastError();                                                        \
        if (e != cudaSuccess)                                                                      \
            return e;                                                                              \
        k_metrics_final<<<1, 256, 0, st>>>(partials, grid, result);                                \
        return cudaGetLastError();                                                                 \
    }
    BTC_MT(1, 1) BTC_MT(2, 1) BTC_MT(4, 1) BTC_MT(8, 1) BTC_MT(16, 1) BTC_MT(32, 1)
    BTC_MT(32, 2)
#undef BTC_MT
    return cudaErrorInvalidValue;
}

template <typename T>
__global__ void k_pack(const double* src, T* dst, long long rows, int R, int Rp)
{
    long long n = rows * Rp;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        long long r = i / Rp;
        int c = (int)(i - r * Rp);
        dst[i] = c < R ? (T)src[r * R + c] : T(0);
    }
}

template <typename T>
__global__ void k_unpack(const T* src, double* dst, long long rows, int R, int Rp)
{
    long long n = rows * R;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        long long r = i / R;
        int c = (int)(i - r * R);
        dst[i] = (double)src[r * Rp + c];
    }
}

__global__ void k_pack_bf16(const double* src, unsigned short* dst, long long rows, int R, int Rp)
{
    long long n = rows * Rp;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        long long r = i / Rp;
        int c = (int)(i - r * Rp);
        dst[i] = c < R ? __bfloat16_as_ushort(__float2bfloat16_rn((float)src[r * R + c])) : (unsigned short)0;
    }
}

__global__ void k_unpack_bf16(const unsigned short* src, double* dst, long long rows, int R, int Rp)
{
    long long n = rows * R;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        long long r = i / R;
        int c = (int)(i - r * R);
        dst[i] = (double)__uint_as_float((unsigned)src[r * Rp + c] << 16);
    }
}

// FP32 master rows of the hot rows: hot_rows[h] is the row of master slot h
__global__ void k_master_pack(const double* src, float* master, const int* hot_rows, int nhot, int R, int Rp)
{
    long long n = (long long)nhot * Rp;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int h = (int)(i / Rp), c = (int)(i - (long long)h * Rp);
        master[i] = c < R ? (float)src[(long long)hot_rows[h] * R + c] : 0.f;
    }
}

__global__ void k_master_unpack(const float* master, double* dst, const int* hot_rows, int nhot, int R, int Rp)
{
    long long n = (long long)nhot * R;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int h = (int)(i / R), c = (int)(i - (long long)h * R);
        dst[(long long)hot_rows[h] * R + c] = (double)master[(long long)h * Rp + c];
    }
}

// BF16 copy of every hot row from its master (round to nearest), so readers of
// the BF16 factors (metrics, export) see the masters' values.
__global__ void k_master_refresh(const float* master, unsigned short* dst, const int* hot_rows, int nhot, int Rp)
{
    long long n = (long long)nhot * Rp;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int h = (int)(i / Rp), c = (int)(i - (long long)h * Rp);
        dst[(long long)hot_rows[h] * Rp + c] = __bfloat16_as_ushort(__float2bfloat16_rn(master[i]));
    }
}

// k_master_refresh for many contexts: blockIdx.y picks the job.
__global__ void k_master_refresh_multi(const RefreshJob* jobs)
{
    const RefreshJob j = jobs[blockIdx.y];
    const long long n = (long long)j.nhot * j.Rp;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int h = (int)(i / j.Rp), c = (int)(i - (long long)h * j.Rp);
        j.bf16[(long long)j.hot_rows[h] * j.Rp + c] = __bfloat16_as_ushort(__float2bfloat16_rn(j.master[i]));
    }
}

__global__ void k_seed_step(unsigned* p) { *p += 0x9E3779B9u; }

int grid_for(long long n)
{
    return (int)std::min<long long>(4096, (n + 255) / 256 + 1);
}

}  // namespace

cudaError_t launch_master_refresh_multi(const RefreshJob* jobs, int njobs, cudaStream_t st)
{
    if (njobs <= 0)
        return cudaSuccess;
    if (njobs > 65535)
        return cudaErrorInvalidValue;
    k_master_refresh_multi<<<dim3(64, njobs), 256, 0, st>>>(jobs);
    return cudaGetLastError();
}

cudaError_t launch_seed_step(unsigned* p, cudaStream_t st)
{
    k_seed_step<<<1, 1, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_master(int op, const double* src, double* dst, float* master, void* bf16, const int* hot_rows,
                          int nhot, int R, int Rp, cudaStream_t st)
{
    if (nhot <= 0)
        return cudaSuccess;
    const int grid = grid_for((long long)nhot * Rp);
    if (op == 0)
        k_master_pack<<<grid, 256, 0, st>>>(src, master, hot_rows, nhot, R, Rp);
    else if (op == 1)
        k_master_unpack<<<grid, 256, 0, st>>>(master, dst, hot_rows, nhot, R, Rp);
    else
        k_master_refresh<<<grid, 256, 0, st>>>(master, (unsigned short*)bf16, hot_rows, nhot, Rp);
    return cudaGetLastError();
}

cudaError_t launch_pack(int dtype, const double* src, void* dst, long long rows, int R, int Rp,
                        cudaStream_t st)
{
    int grid = (int)std::min<long long>(4096, (rows * Rp + 255) / 256 + 1);
    if (dtype == 1)
        k_pack<double><<<grid, 256, 0, st>>>(src, (double*)dst, rows, R, Rp);
    else if (dtype == 0)
        k_pack<float><<<grid, 256, 0, st>>>(src, (float*)dst, rows, R, Rp);
    else if (dtype == 2)
        k_pack_bf16<<<grid, 256, 0, st>>>(src, (unsigned short*)dst, rows, R, Rp);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_unpack(int dtype, const void* src, double* dst, long long rows, int R, int Rp,
                          cudaStream_t st)
{
    int grid = (int)std::min<long long>(4096, (rows * R + 255) / 256 + 1);
    if (dtype == 1)
        k_unpack<double><<<grid, 256, 0, st>>>((const double*)src, dst, rows, R, Rp);
    else if (dtype == 0)
        k_unpack<float><<<grid, 256, 0, st>>>((const float*)src, dst, rows, R, Rp);
    else if (dtype == 2)
        k_unpack_bf16<<<grid, 256, 0, st>>>((const unsigned short*)src, dst, rows, R, Rp);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

int padded_rank(int dtype, int R)
{
    int G, NV;
    if (dtype == 1) {
        pick_shape<double>(R, G, NV);
        return G * NV * 2;
    }
    pick_shape<float>(R, G, NV);
    if (dtype == 2)
        return (G * NV * 4 + 7) / 8 * 8;  // whole 16-byte BF16 chunks
    return G * NV * 4;
}

cudaError_t launch_hogwild(int dtype, const SgdArgs& a, int grid, int block, cudaStream_t st)
{
    if (a.nitems == 0)
        return cudaSuccess;
    if (dtype == 1)
        return hogwild_t<double>(a, grid, block, st);
    if (dtype == 0)
        return hogwild_t<float>(a, grid, block, st);
    return cudaErrorInvalidValue;
}

int hogwild_blocks_per_sm(int dtype, int R, int block)
{
    return dtype == 1 ? hogwild_occ<double>(R, block) : hogwild_occ<float>(R, block);
}

cudaError_t launch_det_wave(int dtype, const int* wave_slots, int n, const SgdArgs& a, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    const int warps = 4;
    const int grid = (n + warps - 1) / warps;
    if (dtype == 1) {
        size_t sm = (size_t)warps * 3 * a.Rp * sizeof(double);
        k_det<double><<<grid, warps * 32, sm, st>>>(wave_slots, n, a);
    } else if (dtype == 0) {
        size_t sm = (size_t)warps * 3 * a.Rp * sizeof(float);
        k_det<float><<<grid, warps * 32, sm, st>>>(wave_slots, n, a);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_lf_wave(int dtype, const int* wave_slots, int n, const SgdArgs& a, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    const int warps = 4;
    const int grid = (n + warps - 1) / warps;
    if (dtype == 1) {
        size_t sm = (size_t)warps * 3 * a.Rp * sizeof(double);
        k_lf<double><<<grid, warps * 32, sm, st>>>(wave_slots, n, a);
    } else if (dtype == 0) {
        size_t sm = (size_t)warps * 3 * a.Rp * sizeof(float);
        k_lf<float><<<grid, warps * 32, sm, st>>>(wave_slots, n, a);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_metrics(int dtype, const int4* coo, const double* val, long long n, const void* A,
                           const void* B, const void* C, int R, int Rp, double* partials, int grid,
                           double* result, cudaStream_t st)
{
    if (dtype == 1)
        return metrics_t<double>(coo, val, n, (const double*)A, (const double*)B, (const double*)C, R,
                                 Rp, partials, grid, result, st);
    if (dtype == 0)
        return metrics_t<float>(coo, val, n, (const float*)A, (const float*)B, (const float*)C, R, Rp,
                                partials, grid, result, st);
    if (dtype == 2)
        return metrics_t<float, unsigned short>(coo, val, n, (const unsigned short*)A,
                                                (const unsigned short*)B, (const unsigned short*)C, R, Rp,
                                                partials, grid, result, st);
    return cudaErrorInvalidValue;
}

}  // namespace btc
