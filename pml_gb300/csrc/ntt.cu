// ntt.cu -- shared-memory NTT kernels (one transform per 1/tpc of a CTA).
//
// Each thread owns 16 residues.  The log2(N) radix-2 stages are processed in
// groups of four (the last forward / first inverse group may be shorter):
// inside a group every thread runs a radix-16 sub-transform in registers.
// Its butterflies only need the constant sixteenth roots of unity; the part of
// the twiddles that depends on the sub-transform's offset factors out of every
// butterfly of the group (it is common to each difference branch) and is
// applied once per residue, after the group for decimation in frequency and
// before it for decimation in time: slot m gets w_span^(off * bitrev4(m)).
// Between groups the residues go through shared memory (padded by one word
// every 16, or 32, against bank conflicts).  Forward transforms are decimation in
// frequency (natural order in, bit-reversed out), inverse ones decimation in
// time (bit-reversed in, natural out): no reordering pass.  Values stay in
// [0, 2q) between forward butterflies and in [0, 4q) between inverse ones
// (q < 2^30, lazy reduction).
#include "ntt.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstring>

namespace pmlg {


// Cache policy: coefficients and evaluations stream through once and are not
// kept in L1 (no_allocate); the group twiddle tables are kept (evict_last).
__device__ __forceinline__ uint64_t ld_stream(const uint64_t *p)
{
    uint64_t v;
    asm("ld.global.nc.L1::no_allocate.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint4 ld_stream(const uint4 *p)
{
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}

__device__ __forceinline__ uint2 ld_keep(const uint2 *p)
{
    uint2 v;
    asm("ld.global.nc.L1::evict_last.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t csub(uint32_t x, uint32_t m) { return min(x, x - m); }

// Radix-2^G decimation-in-frequency butterflies on each of the 16 >> G
// sub-transforms held by a thread, with the constant twiddles
// w_{2^(G-l)}^(m mod half) = c16[(m mod half) * 16 / 2^(G-l)] of stage l.
//
// ZH: the upper half of the input is zero (slot m + 8 of the first group), so
// the first level is v[m + 8] = v[m] * w_16^m and v[m] is unchanged.
// TW: every slot but 0 is multiplied by a group twiddle right after (a Shoup
// product accepts any input below 2^32), so the last level leaves them in
// [0, 4q) instead of reducing them to [0, 2q).
template <int G, bool ZH = false, bool TW = false>
__device__ __forceinline__ void dif_const(uint32_t (&v)[16], const NttDev &T)
{
    constexpr int M = 1 << G, SUB = 16 >> G;
    const uint32_t q = T.q, q2 = 2 * q;
    static_assert(!ZH || G == 4, "zero upper half only in a radix-16 group");
    if constexpr (ZH) {
        v[8] = v[0];
#pragma unroll
        for (int m = 1; m < 8; m++) v[m + 8] = shoup_mul(v[m], T.c16[m], T.c16q[m], q);
    }
#pragma unroll
    for (int u = 0; u < SUB; u++)
#pragma unroll
        for (int l = ZH ? 1 : 0; l < G; l++) {
            const int half = M >> (l + 1);
            const bool last = TW && l == G - 1;
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (m & half) continue;
                const int ti = (m % half) * (16 >> (G - l));
                const uint32_t a = v[u * M + m], b = v[u * M + m + half];
                v[u * M + m] = (last && m != 0) ? a + b : csub(a + b, q2);
                const uint32_t d = a + q2 - b;
                v[u * M + m + half] = last ? d : ti ? shoup_mul(d, T.c16[ti], T.c16q[ti], q) : csub(d, q2);
            }
        }
}

// Radix-2^G decimation-in-time butterflies, constant twiddles
// w_{2^(l+1)}^-(m mod 2^l) = c16[(m mod 2^l) * 16 / 2^(l+1)] (inverse table).
// Lazy in the manner of Harvey: inputs and outputs lie in [0, 4q); only the
// sum operand is brought to [0, 2q) before the butterfly.
template <int G>
__device__ __forceinline__ void dit_const(uint32_t (&v)[16], const NttDev &T)
{
    constexpr int M = 1 << G, SUB = 16 >> G;
    const uint32_t q = T.q, q2 = 2 * q;
#pragma unroll
    for (int u = 0; u < SUB; u++)
#pragma unroll
        for (int l = 0; l < G; l++) {
            const int half = 1 << l;
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (m & half) continue;
                const int ti = (m % half) * (16 >> (l + 1));
                const uint32_t a = csub(v[u * M + m], q2), b = v[u * M + m + half];
                const uint32_t bw = ti ? shoup_mul(b, T.c16[ti], T.c16q[ti], q) : csub(b, q2);
                v[u * M + m] = a + bw;
                v[u * M + m + half] = a + q2 - bw;
            }
        }
}

__device__ __forceinline__ int brev4(int m) { return ((m & 1) << 3) | ((m & 2) << 1) | ((m & 4) >> 1) | ((m & 8) >> 3); }

// Twiddles of a radix-16 group, deferred to one factor per slot: slot m of
// the sub-transform at offset `off` inside blocks of size 2^(lls+4) is
// multiplied by w_span^(off * bitrev4(m)), read from the group table of size
// 2^lls (consecutive offs are consecutive entries: coalesced).
__device__ __forceinline__ void group_twiddles(uint32_t (&v)[16], const NttDev &T, int off, int lls)
{
    const uint2 *g = T.w + 15 * ((1 << lls) - 1) + off;
#pragma unroll
    for (int m = 1; m < 16; m++) {
        const uint2 tw = ld_keep(&g[(m - 1) << lls]);
        v[m] = shoup_mul(v[m], tw.x, tw.y, T.q);
    }
}

// ---------------------------------------------------------------------------
// Kernels, one instantiation per transform size 2^LG: every group's shape is a
// compile-time constant, so the shared-memory exchange is one base address per
// thread plus immediate offsets.  With the padding sidx(i) = i + (i >> PS) (one
// word every 2^PS), the padded index of slot s is sidx(base(t)) + sidx(c_s),
// because c_s is either a multiple of 2^PS or cannot carry the base across one.
// PS = 4 everywhere but in the forward kernels from N = 2^13 on, where one word
// every 32 leaves fewer bank conflicts in the exchanges (2-way ones in the radix-2
// spaced layout instead of the 512- and 32-spaced ones: 512 instead of 768 extra
// wavefronts per transform) and measured 0.1108 against 0.1144 ms per forward
// launch at the headline product; the inverse kernels measured no gain from it.
// ---------------------------------------------------------------------------

template <int LG, int GI>
struct FwdGeom
{
    static constexpr int NG = (LG + 3) / 4;
    static constexpr int G = (GI < NG - 1) ? 4 : LG - 4 * (NG - 1);
    static constexpr int LGH = LG - 1 - 4 * GI;        // log2 of the group's top half size
    static constexpr int LLS = LGH - (G - 1);          // log2 of the sub-transform spacing
    static constexpr int SPAN = 2 << LGH;
};

template <int LG, int GI>
struct InvGeom
{
    static constexpr int NG = (LG + 3) / 4;
    static constexpr int GFIRST = LG - 4 * (NG - 1);
    static constexpr int G = GI == 0 ? GFIRST : 4;
    static constexpr int LLS = GI == 0 ? 0 : GFIRST + 4 * (GI - 1);
    static constexpr int SPAN = 1 << (LLS + G);
};

// padded shared-memory index of slot 0 of thread t in a group (G, LLS, SPAN)
template <int G, int LLS, int SPAN, int PS>
__device__ __forceinline__ int grp_pbase(int t)
{
    if constexpr (G == 4) {
        const int base = (t >> LLS) * SPAN + (t & ((1 << LLS) - 1));
        return base + (base >> PS);
    } else {
        return 16 * t + ((16 * t) >> PS);   // 16 consecutive residues per thread
    }
}

// padded offset of slot s relative to grp_pbase
template <int G, int LLS, int PS>
__device__ __forceinline__ constexpr int grp_poff(int s)
{
    return G == 4 ? (s << LLS) + ((s << LLS) >> PS) : s;
}

// ROT (layouts of 16 consecutive residues per thread, G < 4): register chunk c
// (v[4c .. 4c+3]) holds the residues of slot chunk (c + r) & 3, r = (t >> 1) & 3.  A
// group of at most 2 levels works on aligned runs of 2^G <= 4 slots, so it computes
// the same on rotated registers.  The persistent inverse reads its point tiles (64
// contiguous bytes per thread) in this order: its 16-byte shared-memory loads are then
// conflict-free (in natural order, four lanes of every eight share a bank).  Measured
// on the forward kernel's staging stores as well, the rotation cost more than the
// conflicts it removed (0.122 against 0.115 ms), so only the inverse uses it.
__device__ __forceinline__ int rot_chunk(int t, int c) { return (c + ((t >> 1) & 3)) & 3; }

template <int G, int LLS, int SPAN, int PS, bool ROT = false>
__device__ __forceinline__ void regs_to_smem_t(uint32_t *x, const uint32_t (&v)[16], int t)
{
    uint32_t *p = x + grp_pbase<G, LLS, SPAN, PS>(t);
    if constexpr (ROT) {
        static_assert(G < 4, "rotation of 16 consecutive residues");
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint32_t *pc = p + 4 * rot_chunk(t, c);
#pragma unroll
            for (int u = 0; u < 4; u++) pc[u] = v[4 * c + u];
        }
    } else {
#pragma unroll
        for (int s = 0; s < 16; s++) p[grp_poff<G, LLS, PS>(s)] = v[s];
    }
}

template <int G, int LLS, int SPAN, int PS>
__device__ __forceinline__ void smem_to_regs_t(uint32_t (&v)[16], const uint32_t *x, int t)
{
    const uint32_t *p = x + grp_pbase<G, LLS, SPAN, PS>(t);
#pragma unroll
    for (int s = 0; s < 16; s++) v[s] = p[grp_poff<G, LLS, PS>(s)];
}

// Barriers between groups.  A group reads its layout from shared memory and writes
// its results back in the same layout, so a thread only overwrites words it read
// itself: the one hazard is the next group reading words other threads wrote (one
// barrier per exchange).  From N = 512 on, a layout is warp-local when every warp
// covers the same 512 consecutive residues ([512w, 512w + 512)) in it: the radix-16
// layouts with sub-transforms spaced at most 32 apart, and the 16-consecutive layout
// of a shorter group.  An exchange between two warp-local layouts needs only the
// warp's own barrier.
template <int LG, int G, int LLS>
__device__ __forceinline__ constexpr bool warp_local_layout()
{
    return LG >= 9 && (G < 4 || LLS <= 5);
}

template <int LG, int GI, bool ZH>
__device__ __forceinline__ void fwd_groups(uint32_t (&v)[16], uint32_t *x, int t, const NttDev &T)
{
    if constexpr (GI < FwdGeom<LG, 0>::NG) {
        using Gm = FwdGeom<LG, GI>;
        constexpr bool TW = Gm::G == 4 && Gm::LLS > 0;
        constexpr int PS = LG >= 13 ? 5 : 4;
        if constexpr (GI > 0) {
            using Gp = FwdGeom<LG, GI - 1>;
            if constexpr (warp_local_layout<LG, Gp::G, Gp::LLS>() && warp_local_layout<LG, Gm::G, Gm::LLS>())
                __syncwarp();
            else
                __syncthreads();
            smem_to_regs_t<Gm::G, Gm::LLS, Gm::SPAN, PS>(v, x, t);
        }
        dif_const<Gm::G, ZH && GI == 0, TW>(v, T);
        if constexpr (TW) group_twiddles(v, T, t & ((1 << Gm::LLS) - 1), Gm::LLS);
        if constexpr (GI < Gm::NG - 1) regs_to_smem_t<Gm::G, Gm::LLS, Gm::SPAN, PS>(x, v, t);
        fwd_groups<LG, GI + 1, ZH>(v, x, t, T);
    }
}

// whether the first inverse group is at most radix-4, so that its registers may be
// rotated by whole chunks of four
template <int LG>
__device__ __forceinline__ constexpr bool rot_ok()
{
    return LG >= 12 && InvGeom<LG, 0>::G <= 2;
}

// The first group writes its layout without a barrier: a caller that reuses x for
// another transform separates the last reads of the previous one from it.
// ROT: the registers arrive rotated (see rot_chunk); the first group writes them back
// to their places
template <int LG, int GI, bool ROT = false>
__device__ __forceinline__ void inv_groups(uint32_t (&v)[16], uint32_t *x, int t, const NttDev &T)
{
    if constexpr (GI < InvGeom<LG, 0>::NG) {
        using Gm = InvGeom<LG, GI>;
        if constexpr (GI > 0) {
            using Gp = InvGeom<LG, GI - 1>;
            if constexpr (warp_local_layout<LG, Gp::G, Gp::LLS>() && warp_local_layout<LG, Gm::G, Gm::LLS>())
                __syncwarp();
            else
                __syncthreads();
            smem_to_regs_t<Gm::G, Gm::LLS, Gm::SPAN, 4>(v, x, t);
        }
        if constexpr (Gm::G == 4 && Gm::LLS > 0) group_twiddles(v, T, t & ((1 << Gm::LLS) - 1), Gm::LLS);
        dit_const<Gm::G>(v, T);
        if constexpr (GI < Gm::NG - 1) regs_to_smem_t<Gm::G, Gm::LLS, Gm::SPAN, 4, ROT && GI == 0>(x, v, t);
        inv_groups<LG, GI + 1, false>(v, x, t, T);
    }
}

// Registers per thread the kernels are compiled for (measured on GB300 at
// N = 2^13: the forward transform is fastest at 32, the inverse at 40).
#ifndef PMLG_NTT_FWD_REGS
#define PMLG_NTT_FWD_REGS 32
#endif
#ifndef PMLG_NTT_INV_REGS
#define PMLG_NTT_INV_REGS 40
#endif
#ifndef PMLG_NTT_FWD_TMA
#define PMLG_NTT_FWD_TMA 1       // forward evaluations leave through TMA tensor stores for N >= 4096
#endif
#ifndef PMLG_NTT_INV_TMA
#define PMLG_NTT_INV_TMA 1       // persistent inverse: point tiles brought in by TMA tensor loads
#endif
#ifndef PMLG_NTT_INV_PERSIST
#define PMLG_NTT_INV_PERSIST 1   // persistent, prefetching inverse kernel for N >= 4096
#endif

// threads of a CTA: one transform of N/16 threads, at least 256
template <int LG>
struct NttBlock
{
    static constexpr int TPT = 1 << (LG - 4);
    static constexpr int THREADS = TPT >= 256 ? TPT : 256;
    static constexpr int min_ctas(int regs) { return 65536 / (THREADS * regs) > 0 ? 65536 / (THREADS * regs) : 1; }
    // resident CTAs the kernels ask registers for (per-thread register budgets above)
    static constexpr int FWD_MIN = min_ctas(PMLG_NTT_FWD_REGS);
    static constexpr int INV_MIN = min_ctas(PMLG_NTT_INV_REGS);
    // persistent inverse: shared memory (transform + prefetch) allows 6 / 3 / 1 CTAs;
    // at N = 2^13 two CTAs per SM with 64 registers (no spills) measured 0.136 ms per
    // launch at the headline product against 0.147 for three with 40 (44 bytes spilled)
    static constexpr int INVP_MIN = LG <= 12 ? 6 : LG == 13 ? 2 : 1;
};

// Loads the first group (elements t + m N/16) and runs all groups; with ZH the
// coefficients stop at N/2, so only slots 0..7 are read.
template <int LG, bool ZH>
__device__ __forceinline__ void fwd_transform(uint32_t (&v)[16], uint32_t *x, int t, const NttDev &T,
                                              const NttFwdArgs &a, bool active, int64_t e)
{
    constexpr int TPT = 1 << (LG - 4);
    const uint64_t *src = a.in + (active ? e : 0) * a.in_ld + a.in_off;
    const int L = active ? (int)a.L : 0;
#pragma unroll
    for (int m = 0; m < (ZH ? 8 : 16); m++) {
        const int d = t + m * TPT;
        uint32_t val = 0;
        if (d < L) {
            const uint64_t s = ld_stream(src + d);
            val = a.reduce ? mod64_q(s, T.q, T.r32, T.r32q, T.oneq) : (uint32_t)s;
        }
        v[m] = val;
    }
    fwd_groups<LG, 0, ZH>(v, x, t, T);
}

template <int LG>
__global__ void __launch_bounds__(NttBlock<LG>::THREADS, NttBlock<LG>::FWD_MIN)
ntt_fwd_kernel(NttFwdArgs a, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ uint32_t smem[];
    constexpr int N = 1 << LG, TPT = N >> 4;
    const int tpc = blockDim.x / TPT;
    const int sub = threadIdx.x / TPT, t = threadIdx.x % TPT;
    const int64_t e = (int64_t)blockIdx.x * tpc + sub;
    const int j = blockIdx.y;
    const NttDev &T = a.tab[j];
    uint32_t *x = smem + sub * (N + (N >> 4));
    const bool active = e < a.nent;

    uint32_t v[16];
    if (2 * a.L <= N)
        fwd_transform<LG, true>(v, x, t, T, a, active, e);
    else
        fwd_transform<LG, false>(v, x, t, T, a, active, e);
    // the last group leaves points 16t .. 16t+15 in v[0..15]
    if constexpr (LG >= 12) {
        // One transform per CTA: the evaluations are staged in the exchange buffer
        // (thread t: tiles 4t..4t+3, 64 contiguous bytes) and the tensor-memory
        // accelerator scatters the 16-byte point tiles, 256 tiles per box.
        const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(x);
        if (a.use_tma && (sbase & 127u) == 0) {
            const uint32_t q = T.q;
            __syncthreads();   // every thread is done reading the last layout
            uint4 *stg = reinterpret_cast<uint4 *>(x) + 4 * t;
#pragma unroll
            for (int c = 0; c < 4; c++)
                stg[c] = make_uint4(csub(v[4 * c + 0], q), csub(v[4 * c + 1], q), csub(v[4 * c + 2], q),
                                    csub(v[4 * c + 3], q));
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (threadIdx.x == 0) {
                constexpr int NT = N / kPtTile, NBOX = NT / 256;
                const int z0 = j * NT;
#pragma unroll 1
                for (int b = 0; b < NBOX; b++)
                    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];"
                                 ::"l"(&tmap), "r"(0), "r"((int)e), "r"(z0 + 256 * b),
                                   "r"(sbase + (uint32_t)b * 256u * kPtTile * 4u)
                                 : "memory");
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");   // smem stays live until read
            }
            return;
        }
    }
    if (active) {
        uint32_t *dst = a.out + j * a.prime_stride + e * kPtTile;
        const uint32_t q = T.q;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint4 o;
            o.x = csub(v[4 * c + 0], q); o.y = csub(v[4 * c + 1], q);
            o.z = csub(v[4 * c + 2], q); o.w = csub(v[4 * c + 3], q);
            const int pt = 16 * t + 4 * c;   // first of the four points
            *reinterpret_cast<uint4 *>(dst + (int64_t)(pt / kPtTile) * a.tile_stride + pt % kPtTile) = o;
        }
    }
}

// Output of an inverse transform: element m of thread t is coefficient t + m N/16.
template <int LG>
__device__ __forceinline__ void inv_store(const uint32_t (&v)[16], const NttInvArgs &a, int64_t e, int j, int t,
                                          uint32_t q)
{
    constexpr int TPT = (1 << LG) >> 4;
    // last group: element m of thread t is coefficient t + m * N/16 (the factor
    // 1/N was applied by the pointwise products)
    const int64_t d0 = t - a.lo;
    if (d0 >= 0 && d0 + 15 * TPT < a.cnt) {
        // every slot of this thread is inside [lo, lo + cnt)
        if (a.direct) {
            uint64_t *o = a.out64 + e * a.out_ld + d0;
#pragma unroll
            for (int m = 0; m < 16; m++) o[m * TPT] = csub(csub(v[m], 2 * q), q);
        } else {
            uint32_t *o = a.res32 + (j * a.nent + e) * a.cnt + d0;
#pragma unroll
            for (int m = 0; m < 16; m++) o[m * TPT] = csub(csub(v[m], 2 * q), q);
        }
    } else {
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int64_t d = d0 + m * TPT;
            if (d < 0 || d >= a.cnt) continue;
            const uint32_t val = csub(csub(v[m], 2 * q), q);
            if (a.direct)
                a.out64[e * a.out_ld + d] = val;
            else
                a.res32[(j * a.nent + e) * a.cnt + d] = val;
        }
    }
    if (a.direct)
        for (int64_t d = a.cnt + t; d < a.out_cap; d += TPT) a.out64[e * a.out_ld + d] = 0;
}

template <int LG>
__global__ void __launch_bounds__(NttBlock<LG>::THREADS, NttBlock<LG>::INV_MIN)
ntt_inv_kernel(NttInvArgs a)
{
    extern __shared__ uint32_t smem[];
    constexpr int N = 1 << LG, TPT = N >> 4;
    const int tpc = blockDim.x / TPT;
    const int sub = threadIdx.x / TPT, t = threadIdx.x % TPT;
    const int64_t e = (int64_t)blockIdx.x * tpc + sub;
    const int j = blockIdx.y;
    const NttDev &T = a.tab[j];
    uint32_t *x = smem + sub * (N + (N >> 4));
    const bool active = e < a.nent;

    uint32_t v[16];
    if (active) {
        const uint32_t *src = a.in + j * a.prime_stride + e * kPtTile;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int pt = 16 * t + 4 * c;
            const uint4 o = ld_stream(reinterpret_cast<const uint4 *>(src + (int64_t)(pt / kPtTile) * a.tile_stride +
                                                                     pt % kPtTile));
            v[4 * c + 0] = o.x; v[4 * c + 1] = o.y; v[4 * c + 2] = o.z; v[4 * c + 3] = o.w;
        }
    } else {
#pragma unroll
        for (int m = 0; m < 16; m++) v[m] = 0;
    }
    inv_groups<LG, 0>(v, x, t, T);
    if (active) inv_store<LG>(v, a, e, j, t, T.q);
}

// Persistent inverse transforms, one transform per CTA at a time (N >= 4096):
// while a transform is computed, the point tiles of the CTA's next one are
// already on their way into shared memory (cp.async, 16-byte chunks; each
// thread prefetches and later reads only its own four chunks, so the buffer
// needs no barrier).
template <int LG>
__global__ void __launch_bounds__(NttBlock<LG>::THREADS, NttBlock<LG>::INVP_MIN)
ntt_inv_persist_kernel(NttInvArgs a)
{
    extern __shared__ __align__(16) uint32_t smem[];
    constexpr int N = 1 << LG, TPT = N >> 4;
    static_assert(TPT >= 256, "one transform per CTA");
    uint32_t *x = smem;
    uint32_t *pf = smem + N + (N >> 4);
    const int t = threadIdx.x, j = blockIdx.y;
    const NttDev &T = a.tab[j];
    const uint32_t *base = a.in + j * a.prime_stride;
    // chunk c of thread t sits at 16 t + 4 (c ^ ((t >> 1) & 3)): conflict-free 16-byte reads
    const int sw = (t >> 1) & 3;
    const uint32_t pf_s = (uint32_t)__cvta_generic_to_shared(pf + 16 * t);
    auto prefetch = [&](int64_t ee) {
        const uint32_t *src = base + ee * kPtTile;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int pt = 16 * t + 4 * c;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                         ::"r"(pf_s + 16u * (uint32_t)(c ^ sw)),
                           "l"(src + (int64_t)(pt / kPtTile) * a.tile_stride + pt % kPtTile)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    int64_t e = blockIdx.x;
    if (e < a.nent) prefetch(e);
    for (; e < a.nent; e += gridDim.x) {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        uint32_t v[16];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const uint4 o = *reinterpret_cast<const uint4 *>(pf + 16 * t + 4 * (c ^ sw));
            v[4 * c + 0] = o.x; v[4 * c + 1] = o.y; v[4 * c + 2] = o.z; v[4 * c + 3] = o.w;
        }
        if (e + gridDim.x < a.nent) prefetch(e + gridDim.x);
        __syncthreads();   // the previous transform's last reads of x are done
        inv_groups<LG, 0>(v, x, t, T);
        inv_store<LG>(v, a, e, j, t, T.q);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// The same, with the point tiles brought in by TMA tensor loads (256 tiles per
// box, one transform = N / 1024 boxes) completing on an mbarrier; the wait is
// bounded (on time-out the error word is set and the results are invalid).
// Used up to N = 2^13 (32 KB per transform and mbarrier phase).  At N = 2^14 this
// kernel once returned wrong transforms for about 0.5% of the entries of a
// 2048-entry launch, before the proxy fence below was added (the fence later
// removed the same kind of errors at 2^12 and 2^13); that size has not been
// measured again and keeps the cp.async kernel above.
template <int LG>
__global__ void __launch_bounds__(NttBlock<LG>::THREADS, NttBlock<LG>::INVP_MIN)
ntt_inv_tma_kernel(NttInvArgs a, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) uint32_t smem[];
    constexpr int N = 1 << LG, NT = N / kPtTile, NBOX = NT / 256;
    constexpr uint32_t BYTES = (uint32_t)N * 4u;
    static_assert(BYTES < 65536u, "one mbarrier phase expects less than 64 KB");
    uint32_t *x = smem;
    uint32_t *pf = smem + N + (N >> 4);                 // N + N/16 words: a multiple of 128 bytes
    __shared__ __align__(8) uint64_t bar;
    const int t = threadIdx.x, j = blockIdx.y;
    const NttDev &T = a.tab[j];
    const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(&bar);
    const uint32_t pf_s = (uint32_t)__cvta_generic_to_shared(pf);
    if (pf_s & 127u) {   // a TMA destination must be 128-byte aligned: report and do nothing
        if (t == 0 && a.err) atomicExch(a.err, 1);
        return;
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    __syncthreads();
    auto prefetch = [&](int64_t ee) {   // one thread
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s), "r"(BYTES) : "memory");
#pragma unroll 1
        for (int b = 0; b < NBOX; b++)
            asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                         ::"r"(pf_s + (uint32_t)b * 256u * kPtTile * 4u), "l"(&tmap), "r"(0), "r"((int)ee),
                           "r"(j * NT + 256 * b), "r"(bar_s)
                         : "memory");
    };
    int64_t e = blockIdx.x;
    if (e < a.nent && t == 0) prefetch(e);
    uint32_t phase = 0;
    for (; e < a.nent; e += gridDim.x, phase ^= 1u) {
        uint32_t done = 0;
        unsigned long long t0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        for (int it = 0; it < (1 << 24) && !done; it++) {
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                         : "=r"(done) : "r"(bar_s), "r"(phase) : "memory");
            unsigned long long tn;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tn));
            if (tn - t0 > 500000000ull) break;
        }
        if (!done && a.err) atomicExch(a.err, 1);
        uint32_t v[16];
        constexpr bool ROT = rot_ok<LG>();
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const uint4 o = *reinterpret_cast<const uint4 *>(pf + 16 * t + 4 * (ROT ? rot_chunk(t, c) : c));
            v[4 * c + 0] = o.x; v[4 * c + 1] = o.y; v[4 * c + 2] = o.z; v[4 * c + 3] = o.w;
        }
        // The next TMA load writes this buffer through the async proxy: without a proxy
        // fence after the generic reads, the barrier alone does not order them before it
        // (without the fence, 2 CTAs per SM at N = 2^13 returned a wrong entry in about
        // 1% of the headline products, 4 CTAs per SM at N = 2^12 in 70%).
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();   // the buffer is read: the next transform may come in
        if (t == 0 && done && e + gridDim.x < a.nent) prefetch(e + gridDim.x);
        inv_groups<LG, 0, ROT>(v, x, t, T);
        inv_store<LG>(v, a, e, j, t, T.q);
        if (!__syncthreads_and(done)) break;   // a load that never completed ends the CTA's work
    }
}

// ---------------------------------------------------------------------------

// Garner's CRT of T residues, one instantiation per prime count so the residues and
// the mixed-radix digits stay in registers; every residue of a coefficient is loaded
// before any arithmetic.  The primes are in (2^29.8, 2^30): a Shoup product is below
// 2 q_j and the running value below 2 q_j + 2^30 < 2^32, so the inner Horner steps
// need no reduction, and two conditional subtractions bring it below q_j.  WIDE: p is
// above every prime, so the digits need no reduction mod p.
template <int T, bool WIDE>
__global__ void __launch_bounds__(256)
crt_kernel(CrtPlan plan, const uint32_t *__restrict__ res32, int64_t nent, int64_t cnt,
           uint64_t *__restrict__ out64, int64_t out_ld, int64_t out_cap)
{
    const int64_t plane = nent * cnt;
    // entries along grid y, coefficients along x (no 64-bit division per element)
    for (int64_t e = blockIdx.y; e < nent; e += gridDim.y) {
        const uint32_t *rp = res32 + e * cnt;
        uint64_t *op = out64 + e * out_ld;
        for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < out_cap;
             d += (int64_t)gridDim.x * blockDim.x) {
            if (d >= cnt) {
                op[d] = 0;
                continue;
            }
            uint32_t c[T];
#pragma unroll
            for (int j = 0; j < T; j++) c[j] = __ldg(rp + j * plane + d);
#pragma unroll
            for (int j = 1; j < T; j++) {
                const uint32_t qj = plan.q[j];
                // c_0 + c_1 q_0 + ... + c_{j-1} q_0..q_{j-2} modulo q_j
                uint32_t v = c[j - 1];
#pragma unroll
                for (int l = j - 2; l >= 0; l--) v = shoup_mul(v, plan.qmod[j][l], plan.qmodq[j][l], qj) + c[l];
                v = min(v, v - 2 * qj);
                v = min(v, v - qj);
                const uint32_t diff = c[j] + qj - v;   // in [1, 2 q_j)
                const uint32_t cj = shoup_mul(diff, plan.ginv[j], plan.ginvq[j], qj);
                c[j] = min(cj, cj - qj);
            }
            const uint64_t p = plan.p;
            uint64_t res;
            if (p <= (1ull << 63)) {
                // Horner x <- x q_l + c_l mod p with 64-bit Shoup products (results in [0, 2p))
                auto red = [&](uint64_t v) {   // v < 2^32 -> [0, p)
                    if (WIDE) return v;
                    uint64_t r = v - __umul64hi(v, plan.onepq) * p;
                    return r >= p ? r - p : r;
                };
                uint64_t x = red(c[T - 1]);
#pragma unroll
                for (int l = T - 2; l >= 0; l--) {
                    x = x * plan.qp[l] - __umul64hi(x, plan.qpq[l]) * p;
                    x = x >= p ? x - p : x;
                    const uint64_t s = x + red(c[l]);
                    x = (s < x || s >= p) ? s - p : s;
                }
                res = x;
            } else {
                unsigned __int128 x = c[T - 1] % p;
#pragma unroll
                for (int l = T - 2; l >= 0; l--) x = (x * plan.q[l] + c[l]) % p;
                res = (uint64_t)x;
            }
            op[d] = res;
        }
    }
}

template <int T>
static void crt_launch(const CrtPlan &plan, dim3 grid, const uint32_t *res32, int64_t nent, int64_t cnt,
                       uint64_t *out64, int64_t out_ld, int64_t out_cap, cudaStream_t st)
{
    if (plan.p > (1ull << 30))
        crt_kernel<T, true><<<grid, 256, 0, st>>>(plan, res32, nent, cnt, out64, out_ld, out_cap);
    else
        crt_kernel<T, false><<<grid, 256, 0, st>>>(plan, res32, nent, cnt, out64, out_ld, out_cap);
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

static void ntt_geometry(int lg, int64_t nent, int *threads, int *tpc, size_t *smem, int64_t *blocks)
{
    const int N = 1 << lg, TPT = N >> 4;
    const int th = TPT >= 256 ? TPT : 256;
    *threads = th;
    *tpc = th / TPT;
    *smem = (size_t)(*tpc) * (N + (N >> 4)) * sizeof(uint32_t);
    *blocks = (nent + *tpc - 1) / *tpc;
}

template <int LG>
static cudaError_t set_attrs()
{
    const int sm = (int)(((1 << LG) + (1 << (LG - 4))) * sizeof(uint32_t) * ((1 << (LG - 4)) >= 256 ? 1 : 256 >> (LG - 4)));
    cudaError_t e = cudaFuncSetAttribute(ntt_fwd_kernel<LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ntt_inv_kernel<LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if constexpr (LG >= 12) {
        const int smp = (int)(((1 << LG) + (1 << (LG - 4)) + (1 << LG)) * sizeof(uint32_t));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(ntt_inv_persist_kernel<LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smp);
        if constexpr (LG <= 13)
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(ntt_inv_tma_kernel<LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smp);
    }
    return e;
}

static int ensure_smem_attr(pmlg_ctx *ctx)
{
    static bool done = false;
    if (done) return PMLG_OK;
    PMLG_CUDA_TRY(set_attrs<4>());  PMLG_CUDA_TRY(set_attrs<5>());  PMLG_CUDA_TRY(set_attrs<6>());
    PMLG_CUDA_TRY(set_attrs<7>());  PMLG_CUDA_TRY(set_attrs<8>());  PMLG_CUDA_TRY(set_attrs<9>());
    PMLG_CUDA_TRY(set_attrs<10>()); PMLG_CUDA_TRY(set_attrs<11>()); PMLG_CUDA_TRY(set_attrs<12>());
    PMLG_CUDA_TRY(set_attrs<13>()); PMLG_CUDA_TRY(set_attrs<14>());
    done = true;
    return PMLG_OK;
}

#define NTT_DISPATCH(KERNEL, LGV, GRID, TH, SMEM, ST, ...)                       \
    switch (LGV) {                                                                \
    case 4: KERNEL<4><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;                \
    case 5: KERNEL<5><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;                \
    case 6: KERNEL<6><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;                \
    case 7: KERNEL<7><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;                \
    case 8: KERNEL<8><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;                \
    case 9: KERNEL<9><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;                \
    case 10: KERNEL<10><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;              \
    case 11: KERNEL<11><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;              \
    case 12: KERNEL<12><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;              \
    case 13: KERNEL<13><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;              \
    default: KERNEL<14><<<GRID, TH, SMEM, ST>>>(__VA_ARGS__); break;              \
    }

// cuTensorMapEncodeTiled from the driver, looked up once
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) ==
                cudaSuccess &&
            qr == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

int ntt_forward(pmlg_ctx *ctx, const NttFwdArgs &a0, cudaStream_t st)
{
    if (a0.lg < kMinLgN || a0.lg > kMaxLgN) return PMLG_ELEN;
    if (a0.nent <= 0) return PMLG_OK;
    PMLG_TRY(ensure_smem_attr(ctx));
    int threads, tpc;
    size_t smem;
    int64_t blocks;
    ntt_geometry(a0.lg, a0.nent, &threads, &tpc, &smem, &blocks);
    if (blocks > 0x7fffffffll) return PMLG_EUNSUP;
    NttFwdArgs a = a0;
    // N >= 4096: a 3-D tensor map over the evaluations, (point in tile, entry, tile of any
    // prime), box (kPtTile, 1, 256); without it the kernel stores the tiles itself
    alignas(64) CUtensorMap tmap;
    std::memset(&tmap, 0, sizeof(tmap));
    a.use_tma = 0;
    if (PMLG_NTT_FWD_TMA && a.lg >= 12 && a.nent <= 0x7fffffffll) {
        PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
        const cuuint64_t ntiles = ((cuuint64_t)1 << a.lg) / kPtTile * (cuuint64_t)a.t;
        const cuuint64_t gdim[3] = {(cuuint64_t)kPtTile, (cuuint64_t)a.nent, ntiles};
        const cuuint64_t gstride[2] = {(cuuint64_t)kPtTile * 4u, (cuuint64_t)a.tile_stride * 4u};
        const cuuint32_t box[3] = {(cuuint32_t)kPtTile, 1u, 256u}, estride[3] = {1u, 1u, 1u};
        if (enc && ((uintptr_t)a.out & 15u) == 0 && a.prime_stride == ((int64_t)1 << a.lg) / kPtTile * a.tile_stride &&
            enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, a.out, gdim, gstride, box, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
            a.use_tma = 1;
    }
    prof_begin(ctx, "ntt_fwd", st);
    NTT_DISPATCH(ntt_fwd_kernel, a.lg, dim3((unsigned)blocks, a.t), threads, smem, st, a, tmap);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

int ntt_inverse(pmlg_ctx *ctx, const NttInvArgs &a0, cudaStream_t st)
{
    NttInvArgs a = a0;
    a.err = ctx->d_err;
    if (a.lg < kMinLgN || a.lg > kMaxLgN) return PMLG_ELEN;
    if (a.nent <= 0) return PMLG_OK;
    PMLG_TRY(ensure_smem_attr(ctx));
    int threads, tpc;
    size_t smem;
    int64_t blocks;
    ntt_geometry(a.lg, a.nent, &threads, &tpc, &smem, &blocks);
    if (blocks > 0x7fffffffll) return PMLG_EUNSUP;
    prof_begin(ctx, "ntt_inv", st);
    if (PMLG_NTT_INV_PERSIST && a.lg >= 12) {
        // persistent: as many CTAs as fit on the GPU, each walking over transforms
        const int N = 1 << a.lg;
        const size_t smp = (size_t)(2 * N + (N >> 4)) * sizeof(uint32_t);
        // CTAs launched per SM; at N = 2^13 two are resident, at 2^12 six, and more waves
        // still balance the work better (per 4096-transform launch at 2^13: 0.142 ms with
        // 2 per SM, 0.137 with 3, 0.1345 with 4; at 2^12: 0.0655 with 6, 0.0634 with 12)
        const int per_sm = a.lg == 12 ? 12 : a.lg == 13 ? 4 : 1;
        int64_t g = (int64_t)ctx->sm_count * per_sm;
        if (g > a.nent) g = a.nent;
        const dim3 grid((unsigned)g, a.t);
        // the point tiles come in by TMA when a tensor map over them can be made:
        // (point in tile, entry, tile of any prime), box (kPtTile, 1, 256)
        alignas(64) CUtensorMap tmap;
        std::memset(&tmap, 0, sizeof(tmap));
        bool tma = false;
        if (PMLG_NTT_INV_TMA && a.lg <= 13 && a.nent <= 0x7fffffffll) {
            PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
            const cuuint64_t ntiles = (cuuint64_t)N / kPtTile * (cuuint64_t)a.t;
            const cuuint64_t gdim[3] = {(cuuint64_t)kPtTile, (cuuint64_t)a.nent, ntiles};
            const cuuint64_t gstride[2] = {(cuuint64_t)kPtTile * 4u, (cuuint64_t)a.tile_stride * 4u};
            const cuuint32_t box[3] = {(cuuint32_t)kPtTile, 1u, 256u}, estride[3] = {1u, 1u, 1u};
            tma = enc && ((uintptr_t)a.in & 15u) == 0 && a.prime_stride == (int64_t)N / kPtTile * a.tile_stride &&
                  enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, (void *)a.in, gdim, gstride, box, estride,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        }
        if (tma) {
            if (a.lg == 12)
                ntt_inv_tma_kernel<12><<<grid, N >> 4, smp, st>>>(a, tmap);
            else
                ntt_inv_tma_kernel<13><<<grid, N >> 4, smp, st>>>(a, tmap);
        } else {
            switch (a.lg) {
            case 12: ntt_inv_persist_kernel<12><<<grid, N >> 4, smp, st>>>(a); break;
            case 13: ntt_inv_persist_kernel<13><<<grid, N >> 4, smp, st>>>(a); break;
            default: ntt_inv_persist_kernel<14><<<grid, N >> 4, smp, st>>>(a); break;
            }
        }
    } else {
        NTT_DISPATCH(ntt_inv_kernel, a.lg, dim3((unsigned)blocks, a.t), threads, smem, st, a);
    }
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

int crt_combine(pmlg_ctx *ctx, const CrtPlan &plan, const uint32_t *res32, int64_t nent, int64_t cnt,
                uint64_t *out64, int64_t out_ld, int64_t out_cap, cudaStream_t st)
{
    if (nent <= 0 || out_cap <= 0) return PMLG_OK;
    const int64_t by = nent < 65535 ? nent : 65535;
    int64_t bx = (out_cap + 255) / 256;
    const int64_t cap = ((int64_t)ctx->sm_count * 16 + by - 1) / by;   // about 16 CTAs per SM in all
    if (bx > cap) bx = cap;
    const dim3 grid((unsigned)bx, (unsigned)by);
    prof_begin(ctx, "crt", st);
    switch (plan.t) {
    case 1: crt_launch<1>(plan, grid, res32, nent, cnt, out64, out_ld, out_cap, st); break;
    case 2: crt_launch<2>(plan, grid, res32, nent, cnt, out64, out_ld, out_cap, st); break;
    case 3: crt_launch<3>(plan, grid, res32, nent, cnt, out64, out_ld, out_cap, st); break;
    case 4: crt_launch<4>(plan, grid, res32, nent, cnt, out64, out_ld, out_cap, st); break;
    case 5: crt_launch<5>(plan, grid, res32, nent, cnt, out64, out_ld, out_cap, st); break;
    default: crt_launch<6>(plan, grid, res32, nent, cnt, out64, out_ld, out_cap, st); break;
    }
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

}  // namespace pmlg
