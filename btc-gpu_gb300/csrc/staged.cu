// k_staged: the shared-memory staged SGD kernel.
//
// Persistent CTAs take scheduled slots in schedule order from a global
// counter.  For each tile of the slot's block (see tiles.cpp):
//   1. stage   every distinct row of the tile is copied from L2 into shared
//              memory (snapshot S) with 16-byte ld.cg loads spread over the
//              whole CTA, and a delta buffer D is cleared;
//   2. errors  one lane group per entry: dot of the three staged rows,
//              shuffle-reduced, err = value - dot;
//   3. owners  one lane group per owner segment (a run of <= seg entries
//              sharing a row of one mode) sums err * (other two rows) from S
//              and adds coe*lr*(sum - count*reg*row) into D once;
//   4. write   every staged row's delta goes back to global memory with one
//              vector atomic add per 16 bytes.
// Inside a tile the update is the reference kernel's: all entries of one
// thread_size wave read rows before their deltas land (sgd_Kernel.cu:358-392),
// coe-weighted, L2-regularised per visit.  Tiles of one slot run in order on
// the same CTA; different slots run concurrently and compose additively.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "staged.h"

namespace btc {
namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T>
struct SV;
template <>
struct SV<float> {
    static constexpr int N = 4;
    using V = float4;
};
template <>
struct SV<double> {
    static constexpr int N = 2;
    using V = double2;
};

__device__ __forceinline__ float4 zero_v(float) { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ double2 zero_v(double) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ void red_v(float* p, float4 d) { atomicAdd(reinterpret_cast<float4*>(p), d); }
__device__ __forceinline__ void red_v(double* p, double2 d)
{
    atomicAdd(p, d.x);
    atomicAdd(p + 1, d.y);
}

template <typename T>
__device__ __forceinline__ T tile_value(const int4& q, const double* val64, long long idx);
template <>
__device__ __forceinline__ float tile_value<float>(const int4& q, const double*, long long)
{
    return __int_as_float(q.w);
}
template <>
__device__ __forceinline__ double tile_value<double>(const int4&, const double* val64, long long idx)
{
    return __ldg(val64 + idx);
}

template <typename T, int G, int NV>
__global__ void __launch_bounds__(256) k_staged(StagedArgs a)
{
    using V = typename SV<T>::V;
    constexpr int VN = SV<T>::N;
    constexpr int EPW = 32 / G;
    constexpr int E = NV * VN;
    extern __shared__ __align__(16) unsigned char smem[];
    const int Rp = a.Rp;
    T* S = reinterpret_cast<T*>(smem);
    T* D = S + (size_t)a.cap * Rp;
    int4* ent = reinterpret_cast<int4*>(D + (size_t)a.cap * Rp);
    T* err = reinterpret_cast<T*>(ent + a.wave);
    unsigned short* csr = reinterpret_cast<unsigned short*>(err + a.wave);
    __shared__ int s_slot;

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int sub = lane / G, gl = lane % G;
    T* const FA = static_cast<T*>(a.A);
    T* const FB = static_cast<T*>(a.B);
    T* const FC = static_cast<T*>(a.C);
    const T reg = (T)a.reg;
    const int vpr = Rp / VN;
    const T* coe = static_cast<const T*>(a.slot_coe);

    for (;;) {
        __syncthreads();
        if (tid == 0)
            s_slot = atomicAdd(a.counter, 1);
        __syncthreads();
        const int slot = s_slot;
        if (slot >= a.nslots)
            break;
        const T cx = coe[3 * slot], cy = coe[3 * slot + 1], cz = coe[3 * slot + 2];
        const int t0 = __ldg(&a.slot_tile0[slot]);
        const int t1 = t0 + __ldg(&a.slot_ntiles[slot]);
        for (int t = t0; t < t1; t++) {
            const TileHdr h = a.tiles[t];
            const int nv = h.nrows * vpr;
            const int nxy = h.nx + h.ny;
            // 1. stage rows and clear deltas
            for (int i = tid; i < nv; i += blockDim.x) {
                const int r = i / vpr, c = i - r * vpr;
                const int g = __ldg(&a.rows[h.roff + r]);
                const T* Fm = r < h.nx ? FA : (r < nxy ? FB : FC);
                V v = __ldcg(reinterpret_cast<const V*>(Fm + (size_t)g * Rp) + c);
                reinterpret_cast<V*>(S)[i] = v;
                reinterpret_cast<V*>(D)[i] = zero_v(T(0));
            }
            for (int i = tid; i < h.n; i += blockDim.x)
                ent[i] = __ldcs(&a.ent[h.eoff + i]);
            for (int i = tid; i < 3 * h.n; i += blockDim.x)
                csr[i] = __ldcs(&a.csr[3 * h.eoff + i]);
            __syncthreads();
            // 2. errors
            for (int e0 = warp * EPW; e0 < h.n; e0 += nwarps * EPW) {
                const int e = e0 + sub;
                const bool act = e < h.n;
                T p = T(0);
                int4 q = make_int4(0, 0, 0, 0);
                if (act) {
                    q = ent[e];
                    const T* sx = S + (size_t)(q.x & 0xffff) * Rp;
                    const T* sy = S + (size_t)((unsigned)q.x >> 16) * Rp;
                    const T* sz = S + (size_t)q.y * Rp;
#pragma unroll
                    for (int j = 0; j < NV; j++) {
                        const int o = (j * G + gl) * VN;
                        V vx = *reinterpret_cast<const V*>(sx + o);
                        V vy = *reinterpret_cast<const V*>(sy + o);
                        V vz = *reinterpret_cast<const V*>(sz + o);
                        const T* ax = reinterpret_cast<const T*>(&vx);
                        const T* ay = reinterpret_cast<const T*>(&vy);
                        const T* az = reinterpret_cast<const T*>(&vz);
#pragma unroll
                        for (int k = 0; k < VN; k++)
                            p = fma(ax[k], ay[k] * az[k], p);
                    }
                }
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1)
                    p += __shfl_xor_sync(FULL, p, o);
                if (act && gl == 0)
                    err[e] = tile_value<T>(q, a.val64, h.eoff + e) - p;
            }
            __syncthreads();
            // 3. owner segments
            for (int s0 = warp * EPW; s0 < h.nseg; s0 += nwarps * EPW) {
                const int s = s0 + sub;
                if (s >= h.nseg)
                    continue;
                const int4 sg = __ldg(&a.segs[h.soff + s]);
                const int row = sg.x, m = sg.y, cnt = sg.w;
                const unsigned short* lst = csr + m * h.n + sg.z;
                T acc[E];
#pragma unroll
                for (int i = 0; i < E; i++)
                    acc[i] = T(0);
                for (int k = 0; k < cnt; k++) {
                    const int e = lst[k];
                    const int4 q = ent[e];
                    const int l0 = q.x & 0xffff, l1 = (int)((unsigned)q.x >> 16), l2 = q.y;
                    const int o1 = m == 0 ? l1 : l0;
                    const int o2 = m == 2 ? l1 : l2;
                    const T er = err[e];
                    const T* s1 = S + (size_t)o1 * Rp;
                    const T* s2 = S + (size_t)o2 * Rp;
#pragma unroll
                    for (int j = 0; j < NV; j++) {
                        const int o = (j * G + gl) * VN;
                        V v1 = *reinterpret_cast<const V*>(s1 + o);
                        V v2 = *reinterpret_cast<const V*>(s2 + o);
                        const T* b1 = reinterpret_cast<const T*>(&v1);
                        const T* b2 = reinterpret_cast<const T*>(&v2);
#pragma unroll
                        for (int i = 0; i < VN; i++)
                            acc[j * VN + i] = fma(er, b1[i] * b2[i], acc[j * VN + i]);
                    }
                }
                const T* sr = S + (size_t)row * Rp;
                T* dr = D + (size_t)row * Rp;
                const T w = m == 0 ? cx : (m == 1 ? cy : cz);
                const T creg = (T)cnt * reg;
#pragma unroll
                for (int j = 0; j < NV; j++) {
                    const int o = (j * G + gl) * VN;
#pragma unroll
                    for (int i = 0; i < VN; i++)
                        atomicAdd(dr + o + i, w * (acc[j * VN + i] - creg * sr[o + i]));
                }
            }
            __syncthreads();
            // 4. write back each staged row once
            for (int i = tid; i < nv; i += blockDim.x) {
                const int r = i / vpr, c = i - r * vpr;
                const int g = __ldg(&a.rows[h.roff + r]);
                T* Fm = r < h.nx ? FA : (r < nxy ? FB : FC);
                red_v(Fm + (size_t)g * Rp + c * VN, reinterpret_cast<const V*>(D)[i]);
            }
            __threadfence();
            __syncthreads();
        }
    }
}

template <typename T>
void pick(int R, int& G, int& NV)
{
    constexpr int VN = SV<T>::N;
    NV = 1;
    G = 1;
    while (G * VN < R && G < 32)
        G *= 2;
    while (G * VN * NV < R)
        NV++;
}

template <typename T>
const void* kernel_for(int R)
{
    int G, NV;
    pick<T>(R, G, NV);
#define BTC_KS(g, nv)                                 \
    if (G == g && NV == nv)                           \
        return (const void*)&k_staged<T, g, nv>;
    BTC_KS(1, 1) BTC_KS(2, 1) BTC_KS(4, 1) BTC_KS(8, 1) BTC_KS(16, 1) BTC_KS(32, 1) BTC_KS(32, 2)
#undef BTC_KS
    return nullptr;
}

}  // namespace

size_t staged_smem_bytes(int dtype, int Rp, int cap, int wave)
{
    size_t es = dtype == 1 ? 8 : 4;
    size_t b = 2 * (size_t)cap * Rp * es + (size_t)wave * 16 + (size_t)wave * es + 3 * (size_t)wave * 2;
    return (b + 15) & ~(size_t)15;
}

int staged_cap_for(int dtype, int Rp, int wave, int ctas_per_sm, size_t smem_per_sm, size_t smem_per_block)
{
    size_t es = dtype == 1 ? 8 : 4;
    size_t budget = std::min(smem_per_block, smem_per_sm / (size_t)std::max(1, ctas_per_sm) - 1024);
    size_t fixed = (size_t)wave * (16 + es + 6) + 64;
    if (budget <= fixed)
        return 0;
    return (int)std::min<size_t>(65535, (budget - fixed) / (2 * (size_t)Rp * es));
}

cudaError_t launch_staged(int dtype, const StagedArgs& a, int grid, int block, cudaStream_t st)
{
    const void* fn = dtype == 1 ? kernel_for<double>(a.R) : kernel_for<float>(a.R);
    if (!fn)
        return cudaErrorInvalidValue;
    size_t smem = staged_smem_bytes(dtype, a.Rp, a.cap, a.wave);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    void* args[] = {(void*)&a};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, st);
}

int staged_blocks_per_sm(int dtype, int R, int block, size_t smem)
{
    const void* fn = dtype == 1 ? kernel_for<double>(R) : kernel_for<float>(R);
    if (!fn)
        return 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess)
        return 0;
    return n;
}

}  // namespace btc
