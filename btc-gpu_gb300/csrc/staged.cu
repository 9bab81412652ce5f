// k_staged: the shared-memory staged SGD kernel.
//
// Persistent CTAs take work units (runs of consecutive scheduled slots, in
// schedule order) from a global counter, one unit ahead of the one they work
// on, and walk the tiles of the unit's slots as one stream, fetching each next
// tile's header and staged row ids while the current tile computes.  For each
// tile of the slot's block (see tiles.cpp):
//   1. stage   every distinct row of the tile, its entries and CSR lists are
//              copied from L2 into shared memory (snapshot S) with 16-byte
//              cp.async copies spread over the whole CTA, all in flight at once;
//   2. errors  one lane group per entry: dot of the three staged rows,
//              shuffle-reduced, err = value - dot;
//   3. owners  one lane group per owner segment (a run of <= seg entries
//              sharing a row of one mode; a tile's segments come longest
//              first, so a warp's lane groups run loops of about equal
//              length) sums err * (other two rows) from S
//              in registers and adds coe*lr*(sum - count*reg*row) to the row
//              (row: the snapshot; for a FAST row, its value at write time)
//              in global memory with one vector red per 16 bytes (BF16
//              rows without a master: the stochastically rounded difference
//              to the snapshot, by predicated bf16x2 reds), so a row is
//              written once per segment instead of once per entry.
// Inside a tile the update is the reference kernel's: all entries of one
// thread_size wave read rows before their deltas land (sgd_Kernel.cu:358-392),
// coe-weighted, L2-regularised per visit.  Tiles of one slot run in order on
// the same CTA; different slots run concurrently and compose additively.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "staged.h"

namespace btc {
namespace {

constexpr unsigned FULL = 0xffffffffu;
// Staged row ids: FP32/FP64 rows hold the global row, or ~row for a FAST row
// (decays from its value at write time); BF16 rows hold the global row when
// they have no master, else ~(master index), with bit FAST set in the master
// index for a FAST row.
constexpr int FAST = 1 << 30;

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

// Vector adds to global memory that return nothing (red, not atom): no
// register waits on the old value.
__device__ __forceinline__ void red_v(float* p, float4 d)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(d.x), "f"(d.y), "f"(d.z), "f"(d.w)
                 : "memory");
}
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

// BF16 helpers.  Stochastic rounding follows the published recipe of adding
// uniform random bits below the truncation point and truncating (Gupta et
// al., "Deep Learning with Limited Numerical Precision", 2015): the rounded
// value is unbiased, so updates far below one BF16 ulp still move a row on
// average.  sm_100-family GPUs do it in one instruction per pair,
// cvt.rs.bf16x2.f32 (PTX ISA 8.7): the high half rounds with rbits[31:16],
// the low half with rbits[15:0], up when the 16 discarded mantissa bits plus
// the random bits carry.
__device__ __forceinline__ unsigned mix3(unsigned a, unsigned b, unsigned c)
{
    unsigned h = a * 0x9E3779B1u ^ b * 0x85EBCA77u ^ c * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}
// Word k of rounding bits drawn from a lane's hash h (full avalanche over
// its inputs): a multiply by a distinct odd constant per k, and an
// xor-shift that folds the product's well-mixed high half into its low half.
__device__ __forceinline__ unsigned draw_bits(unsigned h, unsigned k)
{
    const unsigned w = h * (0x9E3779B1u + 0x3C6EF372u * k);
    return w ^ (w >> 16);
}
// {hi, lo} rounded stochastically to a bf16x2 word (hi in bits 31:16)
__device__ __forceinline__ unsigned cvt_rs_bf16x2(float hi, float lo, unsigned rbits)
{
    unsigned d;
    asm("cvt.rs.satfinite.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}
// Adds a - b (bf16x2, rounded to nearest) to the pair at p, fire and
// forget, unless a == b: one predicated red, no branch.
__device__ __forceinline__ void red_bf16x2_diff(void* p, unsigned a, unsigned b)
{
    asm volatile(
        "{\n\t.reg .pred q;\n\t.reg .b32 d;\n\t"
        "setp.ne.b32 q, %1, %2;\n\t"
        "sub.rn.bf16x2 d, %1, %2;\n\t"
        "@q red.global.add.noftz.bf16x2 [%0], d;\n\t}" ::"l"(p),
        "r"(a), "r"(b)
        : "memory");
}
__device__ __forceinline__ float4 bf16x4_to_float4(uint2 raw)
{
    return make_float4(__uint_as_float(raw.x << 16), __uint_as_float(raw.x & 0xffff0000u),
                       __uint_as_float(raw.y << 16), __uint_as_float(raw.y & 0xffff0000u));
}
// One element's update e + (a - c*e): the step with its decay term.
__device__ __forceinline__ float sr_step(float e, float a, float c) { return e + (a - c * e); }

__device__ __forceinline__ float4 ld_bf4(const unsigned short* p)
{
    return bf16x4_to_float4(*reinterpret_cast<const uint2*>(p));
}

// Owner segment packed in one word: local row (bits 0-13), mode (14-15),
// count - 1 (16-19), start in that mode's CSR list (20-31).
__device__ __forceinline__ int seg_row(unsigned s) { return (int)(s & 0x3fffu); }
__device__ __forceinline__ int seg_mode(unsigned s) { return (int)((s >> 14) & 3u); }
__device__ __forceinline__ int seg_count(unsigned s) { return (int)((s >> 16) & 15u) + 1; }
__device__ __forceinline__ int seg_start(unsigned s) { return (int)(s >> 20); }
__device__ __forceinline__ unsigned pack_bf16x2_rn(float lo, float hi)
{
    return (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

__device__ __forceinline__ void cp16(void* smem_dst, const void* gsrc)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// No-op hooks: a tile processed on its own (the batched kernel's path).
struct NoHook {
    __device__ __forceinline__ void after_stage() const {}
    __device__ __forceinline__ void after_errors() const {}
};

// One tile t of slot `slot`: header h, staged row ids in `rid` (already
// filled when rid_ready, else loaded here).  MASK allows a row shorter than
// G*NV*VN elements (the lanes past the padded rank stay idle), so one shape
// serves every rank of a batch.  hook.after_stage() runs once the tile is
// staged and visible to the whole CTA, hook.after_errors() once the errors
// are: a caller uses them to fetch the next tile's header and row ids while
// this tile computes.  fence: the slot's next tile follows on this CTA and
// must see this tile's adds.
template <typename T, int GC, int NV, bool BF, bool MASK, typename Hook>
__device__ __forceinline__ void do_tile(const StagedArgs& a, unsigned char* smem, const TileHdr& h, int t,
                                        int slot, T cx, T cy, T cz, int* rid, bool rid_ready, bool fence,
                                        unsigned seed, const Hook& hook)
{
    using V = typename SV<T>::V;
    constexpr int VN = SV<T>::N;
    // GC > 0: lanes per entry fixed at compile time; GC == 0: taken from the
    // tensor's arguments (a.G, a power of two <= 8) so that a batch of tensors
    // of different ranks keeps every lane busy
    const int G = GC > 0 ? GC : a.G;
    const int EPW = 32 / G;
    constexpr int E = NV * VN;
    const int Rp = a.Rp;
    const StagedLayout L(BF ? 2 : sizeof(T), Rp, a.cap, a.wave);
    T* S = reinterpret_cast<T*>(smem);
    int4* ent = reinterpret_cast<int4*>(smem + L.ent);
    T* err = reinterpret_cast<T*>(smem + L.err);
    unsigned short* csr = reinterpret_cast<unsigned short*>(smem + L.csr);
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int sub = lane / G, gl = lane % G;
    T* const FA = static_cast<T*>(a.A);
    T* const FB = static_cast<T*>(a.B);
    T* const FC = static_cast<T*>(a.C);
    const T reg = (T)a.reg;
    const int vpr = Rp / VN;
    // 16-byte chunks per staged row (BF16 cpr, else vpr) and their log2 when
    // a power of two (-1 otherwise): the staging loops split a chunk index
    // into row and chunk by a shift instead of a division
    const int cpr = Rp / 8;
    const int cps = (cpr & (cpr - 1)) == 0 ? __ffs(cpr) - 1 : -1;
    const int vps = (vpr & (vpr - 1)) == 0 ? __ffs(vpr) - 1 : -1;
    unsigned long long t_start = 0;
    if (a.tile_ns && tid == 0)
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    const int nv = h.nrows * vpr;
    const int nxy = h.nx + h.ny;
    // rounding stream of this visit of this tile (BF16)
    const unsigned tile_bits = BF ? mix3(seed, (unsigned)t, (unsigned)slot) : 0u;
    // the first owner segment of this lane group, fetched now so that
    // its latency hides behind staging and the errors
    const int seg_stride = nwarps * EPW;
    unsigned sg_next = 0;
    if (warp * EPW + sub < h.nseg)
        sg_next = __ldg(&a.segs[h.soff + warp * EPW + sub]);
    // 1. stage: rows, entries and CSR lists, all as 16-byte async copies
    //    (BF16 rows stay BF16; a row with an FP32 master is rounded from it
    //    through registers)
    if constexpr (BF) {
        const int nc = h.nrows * cpr;
        unsigned short* Sb = reinterpret_cast<unsigned short*>(smem);
        for (int i = tid; i < nc; i += blockDim.x) {
            const int r = cps >= 0 ? i >> cps : i / cpr, c = i - r * cpr;
            // the global row, or ~(master index | FAST) for a row with an FP32 master
            // (from shared memory when the caller prefetched it)
            const int g = rid_ready ? rid[r] : __ldg(&a.rows[h.roff + r]);
            const int m = r < h.nx ? 0 : (r < nxy ? 1 : 2);
            if (!rid_ready && c == 0)
                rid[r] = g;
            if (g < 0) {
                const float* mm = m == 0 ? a.master[0] : (m == 1 ? a.master[1] : a.master[2]);
                const size_t hm = (size_t)(~g & (FAST - 1));
                const float4 v0 = __ldcg(reinterpret_cast<const float4*>(mm + hm * Rp + c * 8));
                const float4 v1 = __ldcg(reinterpret_cast<const float4*>(mm + hm * Rp + c * 8 + 4));
                uint4 q;
                q.x = pack_bf16x2_rn(v0.x, v0.y);
                q.y = pack_bf16x2_rn(v0.z, v0.w);
                q.z = pack_bf16x2_rn(v1.x, v1.y);
                q.w = pack_bf16x2_rn(v1.z, v1.w);
                *reinterpret_cast<uint4*>(Sb + (r * Rp + c * 8)) = q;
            } else {
                const unsigned short* Fm = static_cast<const unsigned short*>(
                    m == 0 ? a.A : (m == 1 ? a.B : a.C));
                cp16(Sb + (r * Rp + c * 8), Fm + (size_t)g * Rp + c * 8);
            }
        }
    }
    for (int i = tid; i < (BF ? 0 : nv); i += blockDim.x) {
        const int r = vps >= 0 ? i >> vps : i / vpr, c = i - r * vpr;
        const int g0 = rid_ready ? rid[r] : __ldg(&a.rows[h.roff + r]);  // the global row, or ~row (FAST)
        const int g = g0 < 0 ? ~g0 : g0;
        if constexpr (!BF) {
            if (!rid_ready && c == 0)
                rid[r] = g0;
            const T* Fm = r < h.nx ? FA : (r < nxy ? FB : FC);
            cp16(reinterpret_cast<V*>(S) + i, reinterpret_cast<const V*>(Fm + (size_t)g * Rp) + c);
        }
    }
    for (int i = tid; i < h.n; i += blockDim.x)
        cp16(ent + i, a.ent + h.eoff + i);
    const int nc = (3 * h.n + 7) >> 3;
    for (int i = tid; i < nc; i += blockDim.x)
        cp16(csr + 8 * i, a.csr + h.coff + 8 * i);
    cp_wait_all();
    __syncthreads();
    hook.after_stage();
    // 2. errors
    for (int e0 = warp * EPW; e0 < h.n; e0 += nwarps * EPW) {
        const int e = e0 + sub;
        const bool act = e < h.n;
        T p = T(0);
        int4 q = make_int4(0, 0, 0, 0);
        if (act) {
            q = ent[e];
            // shared-memory offsets in 32-bit arithmetic
            const int rx = (q.x & 0xffff) * Rp, ry = (int)((unsigned)q.x >> 16) * Rp, rz = q.y * Rp;
#pragma unroll
            for (int j = 0; j < NV; j++) {
                const int o = (j * G + gl) * VN;
                if (MASK && o >= Rp)
                    continue;
                V vx, vy, vz;
                if constexpr (BF) {
                    const unsigned short* Sb = reinterpret_cast<const unsigned short*>(smem);
                    vx = ld_bf4(Sb + (rx + o));
                    vy = ld_bf4(Sb + (ry + o));
                    vz = ld_bf4(Sb + (rz + o));
                } else {
                    vx = *reinterpret_cast<const V*>(S + (rx + o));
                    vy = *reinterpret_cast<const V*>(S + (ry + o));
                    vz = *reinterpret_cast<const V*>(S + (rz + o));
                }
                const T* ax = reinterpret_cast<const T*>(&vx);
                const T* ay = reinterpret_cast<const T*>(&vy);
                const T* az = reinterpret_cast<const T*>(&vz);
#pragma unroll
                for (int k = 0; k < VN; k++)
                    p = fma(ax[k], ay[k] * az[k], p);
            }
        }
        for (int o = G / 2; o > 0; o >>= 1)
            p += __shfl_xor_sync(FULL, p, o);
        if (act && gl == 0)
            err[e] = tile_value<T>(q, a.val64, h.eoff + e) - p;
    }
    __syncthreads();
    hook.after_errors();
    // 3. owner segments: reduce in registers, one vector add per 16 bytes
    //    (BF16 without a master: two bf16x2 adds per 4 elements)
    for (int s0 = warp * EPW; s0 < h.nseg; s0 += seg_stride) {
        const int s = s0 + sub;
        const unsigned sg = sg_next;
        if (s + seg_stride < h.nseg)
            sg_next = __ldg(&a.segs[h.soff + s + seg_stride]);
        if (s >= h.nseg)
            continue;
        const int row = seg_row(sg), m = seg_mode(sg), cnt = seg_count(sg);
        const unsigned short* lst = csr + m * h.n + seg_start(sg);
        T acc[E];
#pragma unroll
        for (int i = 0; i < E; i++)
            acc[i] = T(0);
#pragma unroll 2
        for (int k = 0; k < cnt; k++) {
            const int e = lst[k];
            const int4 q = ent[e];
            const int l0 = q.x & 0xffff, l1 = (int)((unsigned)q.x >> 16), l2 = q.y;
            const int o1 = m == 0 ? l1 : l0;
            const int o2 = m == 2 ? l1 : l2;
            const T er = err[e];
            const int r1 = o1 * Rp, r2 = o2 * Rp;
#pragma unroll
            for (int j = 0; j < NV; j++) {
                const int o = (j * G + gl) * VN;
                if (MASK && o >= Rp)
                    continue;
                V v1, v2;
                if constexpr (BF) {
                    const unsigned short* Sb = reinterpret_cast<const unsigned short*>(smem);
                    v1 = ld_bf4(Sb + (r1 + o));
                    v2 = ld_bf4(Sb + (r2 + o));
                } else {
                    v1 = *reinterpret_cast<const V*>(S + (r1 + o));
                    v2 = *reinterpret_cast<const V*>(S + (r2 + o));
                }
                const T* b1 = reinterpret_cast<const T*>(&v1);
                const T* b2 = reinterpret_cast<const T*>(&v2);
#pragma unroll
                for (int i = 0; i < VN; i++)
                    acc[j * VN + i] = fma(er, b1[i] * b2[i], acc[j * VN + i]);
            }
        }
        const T* sr = S + row * Rp;
        const T w = m == 0 ? cx : (m == 1 ? cy : cz);
        const T creg = (T)cnt * reg;
        // Regularisation of a FAST row (one the host found decaying
        // quickly relative to a tile's share of the epoch) takes the
        // row's value at write time, not the tile-start snapshot: such
        // a row is stepped by many concurrent tiles, and a decay
        // computed from a value one tile old is delayed negative
        // feedback whose gain grows with that concurrency until it
        // diverges.  In BF16 every FAST row has a master.
        if constexpr (BF) {
            const int g = rid[row];  // global row, or ~(master index | FAST)
            unsigned short* Fm = static_cast<unsigned short*>(m == 0 ? a.A : (m == 1 ? a.B : a.C));
            // fresh random bits for every rounding: a row without a master
            // is written at most once per tile visit, and a block padded
            // into several slots visits its tiles once per slot, so (epoch
            // seed, mode, slot, tile, row, lane, vector) names one update.
            // Bits reused across the updates of an epoch would round an
            // element the same way every time and let its magnitude drift by
            // up to one ulp per update.
            const unsigned hl = g >= 0 ? mix3(tile_bits ^ (unsigned)(m * 0x68E31DA4u), (unsigned)g, (unsigned)gl) : 0u;
#pragma unroll
            for (int j = 0; j < NV; j++) {
                const int o = (j * G + gl) * VN;
                if (MASK && o >= Rp)
                    continue;
                const float wc = w * creg;
                const float4 wa = make_float4(w * acc[j * VN + 0], w * acc[j * VN + 1],
                                              w * acc[j * VN + 2], w * acc[j * VN + 3]);
                const uint2 raw = *reinterpret_cast<const uint2*>(
                    reinterpret_cast<const unsigned short*>(smem) + (row * Rp + o));
                if (g < 0) {
                    float* mp = (m == 0 ? a.master[0] : (m == 1 ? a.master[1] : a.master[2])) +
                                (size_t)(~g & (FAST - 1)) * Rp + o;
                    const float4 base = (~g & FAST) ? __ldcg(reinterpret_cast<const float4*>(mp))
                                                    : bf16x4_to_float4(raw);
                    red_v(mp, make_float4(wa.x - wc * base.x, wa.y - wc * base.y, wa.z - wc * base.z,
                                          wa.w - wc * base.w));
                } else {
                    // The new value is computed from the snapshot and rounded
                    // stochastically; its difference to the snapshot (a few
                    // ulps, exact in BF16) lands by fire-and-forget bf16x2
                    // atomic adds, skipped when the rounding left the pair
                    // unchanged (always so for a zero step on a zero row).
                    // With no other tile on the row since the snapshot the
                    // result is exactly the rounded value.
                    unsigned short* wp = Fm + (size_t)g * Rp + o;
                    const float4 own = bf16x4_to_float4(raw);
                    const unsigned n01 = cvt_rs_bf16x2(sr_step(own.y, wa.y, wc), sr_step(own.x, wa.x, wc),
                                                       draw_bits(hl, 2u * j));
                    const unsigned n23 = cvt_rs_bf16x2(sr_step(own.w, wa.w, wc), sr_step(own.z, wa.z, wc),
                                                       draw_bits(hl, 2u * j + 1u));
                    red_bf16x2_diff(wp, n01, raw.x);
                    red_bf16x2_diff(wp + 2, n23, raw.y);
                }
            }
        } else {
            const int v = rid[row];  // global row, or ~row (FAST)
            T* gr = (m == 0 ? FA : (m == 1 ? FB : FC)) + (size_t)(v < 0 ? ~v : v) * Rp;
#pragma unroll
            for (int j = 0; j < NV; j++) {
                const int o = (j * G + gl) * VN;
                if (MASK && o >= Rp)
                    continue;
                V d;
                T* dd = reinterpret_cast<T*>(&d);
                if (v < 0) {
                    const V cur = __ldcg(reinterpret_cast<const V*>(gr + o));
                    const T* cc = reinterpret_cast<const T*>(&cur);
#pragma unroll
                    for (int i = 0; i < VN; i++)
                        dd[i] = w * (acc[j * VN + i] - creg * cc[i]);
                } else {
#pragma unroll
                    for (int i = 0; i < VN; i++)
                        dd[i] = w * (acc[j * VN + i] - creg * sr[o + i]);
                }
                red_v(gr + o, d);
            }
        }
    }
    // the slot's next tile must see these adds (nothing orders the
    // adds of different slots, so the last tile needs no fence)
    if (fence)
        __threadfence();
    __syncthreads();
        if (a.tile_ns && tid == 0) {
            unsigned long long t_end;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
            a.tile_ns[t] = (unsigned)min(t_end - t_start, 0xffffffffull);
        }
}

// One work unit of one tensor: slots [unit_off[unit], unit_off[unit+1]),
// tile by tile.
template <typename T, int GC, int NV, bool BF, bool MASK>
__device__ __forceinline__ void run_unit(const StagedArgs& a, int unit, unsigned char* smem)
{
    const StagedLayout L(BF ? 2 : sizeof(T), a.Rp, a.cap, a.wave);
    int* rid = reinterpret_cast<int*>(smem + L.rid);
    const T* coe = static_cast<const T*>(a.slot_coe);
    const unsigned seed = a.seed_ptr ? (a.seed ^ *a.seed_ptr) : a.seed;
    const int u0 = __ldg(&a.unit_off[unit]), u1 = __ldg(&a.unit_off[unit + 1]);
    for (int slot = u0; slot < u1; slot++) {
        const T cx = coe[3 * slot], cy = coe[3 * slot + 1], cz = coe[3 * slot + 2];
        const int t0 = __ldg(&a.slot_tile0[slot]);
        const int t1 = t0 + __ldg(&a.slot_ntiles[slot]);
        for (int t = t0; t < t1; t++) {
            const TileHdr h = a.tiles[t];
            do_tile<T, GC, NV, BF, MASK>(a, smem, h, t, slot, cx, cy, cz, rid, false, t + 1 < t1, seed, NoHook());
        }
    }
}

// A CTA's place in its stream of tiles: work unit, slot, tile, the slot's
// tile end (tile < 0: the stream has ended).
struct Pos {
    int unit, slot, t, t_end;
};

// The first tile of unit u at or after slot `slot`, skipping slots whose
// block has no entries (no tiles); t = -1 when the unit has none left.
__device__ __forceinline__ Pos slot_pos(const StagedArgs& a, int u, int slot)
{
    const int s1 = __ldg(&a.unit_off[u + 1]);
    for (; slot < s1; slot++) {
        const int n = __ldg(&a.slot_ntiles[slot]);
        if (n > 0) {
            const int t = __ldg(&a.slot_tile0[slot]);
            return Pos{u, slot, t, t + n};
        }
    }
    return Pos{u, s1, -1, -1};
}

// The first tile of the unit taken ahead (*ahead), which is replaced by a new
// one from the counter; units without tiles are passed over.  t = -1 once the
// units are exhausted.
__device__ __forceinline__ Pos unit_pos(const StagedArgs& a, int* ahead)
{
    for (;;) {
        const int u = *ahead;
        if (u >= a.nunits)
            return Pos{u, 0, -1, -1};
        *ahead = atomicAdd(a.counter, 1);
        const Pos p = slot_pos(a, u, __ldg(&a.unit_off[u]));
        if (p.t >= 0)
            return p;
    }
}

// The tile after p: the slot's next tile, else the first tile of the unit's
// next slot that has tiles, else the first tile of the next unit.
__device__ __forceinline__ Pos next_pos(const StagedArgs& a, Pos p, int* ahead)
{
    if (p.t + 1 < p.t_end) {
        p.t++;
        return p;
    }
    const Pos q = slot_pos(a, p.unit, p.slot + 1);
    return q.t >= 0 ? q : unit_pos(a, ahead);
}

// Loads the next tile's header (after the current tile is staged) and its
// staged row ids (after the current tile's errors), so that the next tile's
// row copies start without waiting on either.
struct Ahead {
    const StagedArgs* a;
    const Pos* pos;   // the next tile's position (shared)
    TileHdr* hdr;     // its header slot (shared)
    int* rid;         // its row-id buffer (shared)
    __device__ __forceinline__ void after_stage() const
    {
        if (threadIdx.x < 4 && pos->t >= 0)
            reinterpret_cast<int4*>(hdr)[threadIdx.x] = __ldg(reinterpret_cast<const int4*>(a->tiles + pos->t) +
                                                              threadIdx.x);
    }
    __device__ __forceinline__ void after_errors() const
    {
        if (pos->t < 0)
            return;
        const int n = hdr->nrows;
        const int* src = a->rows + hdr->roff;
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            rid[i] = __ldg(src + i);
    }
};

// The single-tensor kernel: every CTA walks its stream of tiles -- work
// units taken from the counter one ahead, their slots, the slots' tiles --
// and fetches each next tile's header and row ids while the current tile
// computes (two buffers each in shared memory).
template <typename T, int G, int NV, bool BF>
__global__ void __launch_bounds__(256, 4) k_staged(StagedArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Pos s_pos[2];
    __shared__ int s_ahead;
    const StagedLayout L(BF ? 2 : sizeof(T), a.Rp, a.cap, a.wave);
    TileHdr* hdr = reinterpret_cast<TileHdr*>(smem + L.hdr);
    int* const rid0 = reinterpret_cast<int*>(smem + L.rid);
    int* const rid1 = reinterpret_cast<int*>(smem + L.rid2);
    const T* coe = static_cast<const T*>(a.slot_coe);
    const unsigned seed = a.seed_ptr ? (a.seed ^ *a.seed_ptr) : a.seed;
    if (threadIdx.x == 0) {
        s_ahead = atomicAdd(a.counter, 1);
        s_pos[0] = unit_pos(a, &s_ahead);
    }
    __syncthreads();
    if (s_pos[0].t < 0)
        return;
    // the first tile's header and row ids, fetched in place
    if (threadIdx.x < 4)
        reinterpret_cast<int4*>(hdr)[threadIdx.x] = __ldg(reinterpret_cast<const int4*>(a.tiles + s_pos[0].t) +
                                                          threadIdx.x);
    __syncthreads();
    for (int i = threadIdx.x; i < hdr[0].nrows; i += blockDim.x)
        rid0[i] = __ldg(a.rows + hdr[0].roff + i);
    __syncthreads();
    int cur = 0, cur_slot = -1;
    T cx = T(0), cy = T(0), cz = T(0);
    for (;;) {
        const Pos p = s_pos[cur];
        if (p.t < 0)
            break;
        const int nxt = cur ^ 1;
        // published by the tile's first barrier, before any thread reads it
        if (threadIdx.x == 0)
            s_pos[nxt] = next_pos(a, p, &s_ahead);
        if (p.slot != cur_slot) {
            cx = coe[3 * p.slot];
            cy = coe[3 * p.slot + 1];
            cz = coe[3 * p.slot + 2];
            cur_slot = p.slot;
        }
        const TileHdr h = hdr[cur];
        const Ahead hook{&a, &s_pos[nxt], &hdr[nxt], nxt ? rid1 : rid0};
        do_tile<T, G, NV, BF, false>(a, smem, h, p.t, p.slot, cx, cy, cz, cur ? rid1 : rid0, true, p.t + 1 < p.t_end,
                                     seed, hook);
        cur = nxt;
    }
}

// Many tensors in one persistent launch: work items (tensor, unit) are taken
// from one counter; each tensor brings its own arguments (rank, tiles,
// factors, weights, lanes per entry).  Up to 8 lanes per entry and 4 vectors
// per lane: ranks up to 128 (FP32/BF16).
template <bool BF>
__global__ void __launch_bounds__(256, 4) k_staged_multi(const StagedArgs* __restrict__ tensors,
                                                         const int2* __restrict__ items, int nitems, int* counter)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_item;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0)
            s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems)
            break;
        const int2 w = __ldg(&items[it]);
        const StagedArgs a = tensors[w.x];
        run_unit<float, 0, 4, BF, true>(a, w.y, smem);
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

template <typename T, bool BF>
const void* kernel_for(int R, int G, int NV)
{
    if (G <= 0)
        pick<T>(R, G, NV);
#define BTC_KS(g, nv)                                 \
    if (G == g && NV == nv)                           \
        return (const void*)&k_staged<T, g, nv, BF>;
    BTC_KS(1, 1) BTC_KS(2, 1) BTC_KS(4, 1) BTC_KS(8, 1) BTC_KS(16, 1) BTC_KS(32, 1) BTC_KS(32, 2)
    BTC_KS(1, 2) BTC_KS(2, 2) BTC_KS(4, 2) BTC_KS(8, 2) BTC_KS(16, 2)
#undef BTC_KS
    return nullptr;
}

const void* kernel_for_dtype(int dtype, int R, int G, int NV)
{
    if (dtype == 1)
        return kernel_for<double, false>(R, G, NV);
    if (dtype == 2)
        return kernel_for<float, true>(R, G, NV);
    return kernel_for<float, false>(R, G, NV);
}

}  // namespace

size_t staged_smem_bytes(int dtype, int Rp, int cap, int wave)
{
    return StagedLayout(dtype == 1 ? 8 : (dtype == 2 ? 2 : 4), Rp, cap, wave).total;
}

int staged_cap_for(int dtype, int Rp, int wave, int ctas_per_sm, size_t smem_per_sm, size_t smem_per_block)
{
    size_t es = dtype == 1 ? 8 : (dtype == 2 ? 2 : 4);
    // per CTA the SM reserves 1 KB, and the kernels' static shared
    // variables (work positions, <= 64 bytes) come on top of the dynamic
    // layout: a layout that filled the rest would cost one resident CTA
    size_t budget = std::min(smem_per_block - 128, smem_per_sm / (size_t)std::max(1, ctas_per_sm) - 1024 - 128);
    int cap = (int)std::min<size_t>(16383, budget / ((size_t)Rp * es + 4));
    while (cap > 0 && staged_smem_bytes(dtype, Rp, cap, wave) > budget)
        cap--;
    return cap;
}

int staged_vector_width(int dtype) { return dtype == 1 ? 2 : 4; }

void staged_default_shape(int dtype, int R, int* G, int* NV)
{
    if (dtype == 1)
        pick<double>(R, *G, *NV);
    else
        pick<float>(R, *G, *NV);
}

bool staged_shape_exists(int dtype, int R, int G, int NV)
{
    return G > 0 && kernel_for_dtype(dtype, R, G, NV) != nullptr;
}

cudaError_t launch_staged_multi(int dtype, const StagedArgs* tensors, const int2* items, int nitems, int* counter,
                                size_t smem, int grid, cudaStream_t st)
{
    const void* fn = dtype == 2 ? (const void*)&k_staged_multi<true> : (const void*)&k_staged_multi<false>;
    if (dtype == 1)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    void* args[] = {(void*)&tensors, (void*)&items, (void*)&nitems, (void*)&counter};
    return cudaLaunchKernel(fn, dim3(grid), dim3(256), args, smem, st);
}

int staged_multi_blocks_per_sm(int dtype, size_t smem)
{
    const void* fn = dtype == 2 ? (const void*)&k_staged_multi<true> : (const void*)&k_staged_multi<false>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, 256, smem) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_staged(int dtype, const StagedArgs& a, int grid, int block, cudaStream_t st)
{
    const void* fn = kernel_for_dtype(dtype, a.R, a.G, a.NV);
    if (!fn)
        return cudaErrorInvalidValue;
    size_t smem = staged_smem_bytes(dtype, a.Rp, a.cap, a.wave);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    void* args[] = {(void*)&a};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, st);
}

int staged_blocks_per_sm_shape(int dtype, int R, int G, int NV, int block, size_t smem)
{
    const void* fn = kernel_for_dtype(dtype, R, G, NV);
    if (!fn)
        return 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess)
        return 0;
    return n;
}

int staged_blocks_per_sm(int dtype, int R, int block, size_t smem)
{
    const void* fn = kernel_for_dtype(dtype, R, 0, 0);
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
