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
// every 16 against bank conflicts).  Forward transforms are decimation in
// frequency (natural order in, bit-reversed out), inverse ones decimation in
// time (bit-reversed in, natural out): no reordering pass.  Values stay in
// [0, 2q) between butterflies (q < 2^30, lazy reduction).
#include "ntt.cuh"

namespace pmlg {

__device__ __forceinline__ int sidx(int i) { return i + (i >> 4); }

// Index of register slot (u, m) for a thread t in a group whose sub-transforms
// have 2^G elements spaced 2^lls apart inside blocks of `span`.
__device__ __forceinline__ int grp_index(int t, int u, int m, int G, int lls, int span)
{
    const int sub = 16 >> G;
    const int sp = t * sub + u;
    const int blk = sp >> lls;
    const int off = sp & ((1 << lls) - 1);
    return blk * span + off + (m << lls);
}

__device__ __forceinline__ uint32_t csub(uint32_t x, uint32_t m) { return min(x, x - m); }

// Radix-2^G decimation-in-frequency butterflies on each of the 16 >> G
// sub-transforms held by a thread, with the constant twiddles
// w_{2^(G-l)}^(m mod half) = c16[(m mod half) * 16 / 2^(G-l)] of stage l.
template <int G>
__device__ __forceinline__ void dif_const(uint32_t (&v)[16], const NttDev &T)
{
    constexpr int M = 1 << G, SUB = 16 >> G;
    const uint32_t q = T.q, q2 = 2 * q;
#pragma unroll
    for (int u = 0; u < SUB; u++)
#pragma unroll
        for (int l = 0; l < G; l++) {
            const int half = M >> (l + 1);
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (m & half) continue;
                const int ti = (m % half) * (16 >> (G - l));
                const uint32_t a = v[u * M + m], b = v[u * M + m + half];
                v[u * M + m] = csub(a + b, q2);
                const uint32_t d = a + q2 - b;
                v[u * M + m + half] = ti ? shoup_mul(d, T.c16[ti], T.c16q[ti], q) : csub(d, q2);
            }
        }
}

// Radix-2^G decimation-in-time butterflies, constant twiddles
// w_{2^(l+1)}^-(m mod 2^l) = c16[(m mod 2^l) * 16 / 2^(l+1)] (inverse table).
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
                const uint32_t a = v[u * M + m], b = v[u * M + m + half];
                const uint32_t bw = ti ? shoup_mul(b, T.c16[ti], T.c16q[ti], q) : b;
                v[u * M + m] = csub(a + bw, q2);
                v[u * M + m + half] = csub(a + q2 - bw, q2);
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
        const uint2 tw = __ldg(&g[(m - 1) << lls]);
        v[m] = shoup_mul(v[m], tw.x, tw.y, T.q);
    }
}

__device__ __forceinline__ void regs_to_smem(uint32_t *x, const uint32_t (&v)[16], int t, int G, int lls, int span)
{
#pragma unroll
    for (int s = 0; s < 16; s++) x[sidx(grp_index(t, s >> G, s & ((1 << G) - 1), G, lls, span))] = v[s];
}

__device__ __forceinline__ void smem_to_regs(uint32_t (&v)[16], const uint32_t *x, int t, int G, int lls, int span)
{
#pragma unroll
    for (int s = 0; s < 16; s++) v[s] = x[sidx(grp_index(t, s >> G, s & ((1 << G) - 1), G, lls, span))];
}

// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(1024)
ntt_fwd_kernel(NttFwdArgs a)
{
    extern __shared__ uint32_t smem[];
    const int lg = a.lg, N = 1 << lg, TPT = N >> 4;
    const int tpc = blockDim.x >> (lg - 4);
    const int sub = threadIdx.x >> (lg - 4), t = threadIdx.x & (TPT - 1);
    const int64_t e = (int64_t)blockIdx.x * tpc + sub;
    const int j = blockIdx.y;
    const NttDev &T = a.tab[j];
    uint32_t *x = smem + sub * (N + (N >> 4));
    const bool active = e < a.nent;

    // first group: elements t + m * N/16
    uint32_t v[16];
    {
        const uint64_t *src = a.in + (active ? e : 0) * a.in_ld + a.in_off;
        const int L = active ? (int)a.L : 0;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int d = t + m * TPT;
            uint32_t val = 0;
            if (d < L) {
                const uint64_t s = src[d];
                val = a.reduce ? mod64_q(s, T.q, T.r32, T.r32q, T.oneq) : (uint32_t)s;
            }
            v[m] = val;
        }
    }
    const int ngroups = (lg + 3) >> 2;
    int lgH = lg - 1;
    for (int gi = 0; gi < ngroups; gi++) {
        const int G = (gi < ngroups - 1) ? 4 : lg - 4 * (ngroups - 1);
        const int lls = lgH - (G - 1), span = 2 << lgH;
        if (gi > 0) {
            __syncthreads();
            smem_to_regs(v, x, t, G, lls, span);
        }
        if (G == 4) {
            dif_const<4>(v, T);
            if (lls > 0) group_twiddles(v, T, t & ((1 << lls) - 1), lls);
        } else if (G == 3) {
            dif_const<3>(v, T);
        } else if (G == 2) {
            dif_const<2>(v, T);
        } else {
            dif_const<1>(v, T);
        }
        if (gi < ngroups - 1) {
            __syncthreads();   // everyone done reading the previous layout
            regs_to_smem(x, v, t, G, lls, span);
        }
        lgH -= G;
    }
    // the last group leaves points 16t .. 16t+15 in v[0..15]
    if (active) {
        uint32_t *dst = a.out + j * a.prime_stride + e * kPtTile;
        const uint32_t q = T.q;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint4 o;
            o.x = csub(v[4 * c + 0], q); o.y = csub(v[4 * c + 1], q);
            o.z = csub(v[4 * c + 2], q); o.w = csub(v[4 * c + 3], q);
            *reinterpret_cast<uint4 *>(dst + (int64_t)(4 * t + c) * a.tile_stride) = o;
        }
    }
}

__global__ void __launch_bounds__(1024)
ntt_inv_kernel(NttInvArgs a)
{
    extern __shared__ uint32_t smem[];
    const int lg = a.lg, N = 1 << lg, TPT = N >> 4;
    const int tpc = blockDim.x >> (lg - 4);
    const int sub = threadIdx.x >> (lg - 4), t = threadIdx.x & (TPT - 1);
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
            const uint4 o = *reinterpret_cast<const uint4 *>(src + (int64_t)(4 * t + c) * a.tile_stride);
            v[4 * c + 0] = o.x; v[4 * c + 1] = o.y; v[4 * c + 2] = o.z; v[4 * c + 3] = o.w;
        }
    } else {
#pragma unroll
        for (int m = 0; m < 16; m++) v[m] = 0;
    }
    const int ngroups = (lg + 3) >> 2;
    const int Gfirst = lg - 4 * (ngroups - 1);
    int lls = 0;
    for (int gi = 0; gi < ngroups; gi++) {
        const int G = (gi == 0) ? Gfirst : 4;
        const int span = 1 << (lls + G);
        if (gi > 0) {
            __syncthreads();
            smem_to_regs(v, x, t, G, lls, span);
        }
        if (G == 4) {
            if (lls > 0) group_twiddles(v, T, t & ((1 << lls) - 1), lls);
            dit_const<4>(v, T);
        } else if (G == 3) {
            dit_const<3>(v, T);
        } else if (G == 2) {
            dit_const<2>(v, T);
        } else {
            dit_const<1>(v, T);
        }
        if (gi < ngroups - 1) {
            __syncthreads();
            regs_to_smem(x, v, t, G, lls, span);
        }
        lls += G;
    }
    // last group: element m of thread t is coefficient t + m * N/16
    if (!active) return;
#pragma unroll
    for (int m = 0; m < 16; m++) {
        const int64_t d = t + m * TPT - a.lo;
        if (d < 0 || d >= a.cnt) continue;
        const uint32_t val = csub(shoup_mul(v[m], T.ninv, T.ninvq, T.q), T.q);
        if (a.direct)
            a.out64[e * a.out_ld + d] = val;
        else
            a.res32[(j * a.nent + e) * a.cnt + d] = val;
    }
    if (a.direct)
        for (int64_t d = a.cnt + t; d < a.out_cap; d += TPT) a.out64[e * a.out_ld + d] = 0;
}

// ---------------------------------------------------------------------------

__global__ void crt_kernel(CrtPlan plan, const uint32_t *__restrict__ res32, int64_t nent, int64_t cnt,
                           uint64_t *__restrict__ out64, int64_t out_ld, int64_t out_cap)
{
    const int64_t total = nent * out_cap;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx / out_cap, d = idx - e * out_cap;
        if (d >= cnt) {
            out64[e * out_ld + d] = 0;
            continue;
        }
        uint32_t c[kMaxPrimes];
        c[0] = res32[e * cnt + d];
        for (int j = 1; j < plan.t; j++) {
            const uint32_t qj = plan.q[j];
            // value of c_0 + c_1 q_0 + ... + c_{j-1} q_0..q_{j-2} modulo q_j
            uint32_t v = c[j - 1];
            for (int l = j - 2; l >= 0; l--) {
                v = v >= qj ? v - qj : v;
                v = shoup_mul(v, plan.qmod[j][l], plan.qmodq[j][l], qj) + c[l];   // < 2 qj + 2^30
                while (v >= qj) v -= qj;
            }
            while (v >= qj) v -= qj;
            const uint32_t r = res32[(j * nent + e) * cnt + d];
            uint32_t diff = r >= v ? r - v : r + qj - v;
            uint32_t cj = shoup_mul(diff, plan.ginv[j], plan.ginvq[j], qj);
            c[j] = cj >= qj ? cj - qj : cj;
        }
        const uint64_t p = plan.p;
        unsigned __int128 x = c[plan.t - 1] % p;
        for (int l = plan.t - 2; l >= 0; l--) x = (x * plan.q[l] + c[l]) % p;
        out64[e * out_ld + d] = (uint64_t)x;
    }
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

static int ensure_smem_attr(pmlg_ctx *ctx)
{
    static bool done = false;
    if (done) return PMLG_OK;
    const int maxsm = (int)(((1 << kMaxLgN) + (1 << (kMaxLgN - 4))) * sizeof(uint32_t)) * 1;
    PMLG_CUDA_TRY(cudaFuncSetAttribute(ntt_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm + 4096));
    PMLG_CUDA_TRY(cudaFuncSetAttribute(ntt_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm + 4096));
    done = true;
    return PMLG_OK;
}

int ntt_forward(pmlg_ctx *ctx, const NttFwdArgs &a, cudaStream_t st)
{
    if (a.lg < kMinLgN || a.lg > kMaxLgN) return PMLG_ELEN;
    if (a.nent <= 0) return PMLG_OK;
    PMLG_TRY(ensure_smem_attr(ctx));
    int threads, tpc;
    size_t smem;
    int64_t blocks;
    ntt_geometry(a.lg, a.nent, &threads, &tpc, &smem, &blocks);
    if (blocks > 0x7fffffffll) return PMLG_EUNSUP;
    prof_begin(ctx, "ntt_fwd", st);
    ntt_fwd_kernel<<<dim3((unsigned)blocks, a.t), threads, smem, st>>>(a);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

int ntt_inverse(pmlg_ctx *ctx, const NttInvArgs &a, cudaStream_t st)
{
    if (a.lg < kMinLgN || a.lg > kMaxLgN) return PMLG_ELEN;
    if (a.nent <= 0) return PMLG_OK;
    PMLG_TRY(ensure_smem_attr(ctx));
    int threads, tpc;
    size_t smem;
    int64_t blocks;
    ntt_geometry(a.lg, a.nent, &threads, &tpc, &smem, &blocks);
    if (blocks > 0x7fffffffll) return PMLG_EUNSUP;
    prof_begin(ctx, "ntt_inv", st);
    ntt_inv_kernel<<<dim3((unsigned)blocks, a.t), threads, smem, st>>>(a);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

int crt_combine(pmlg_ctx *ctx, const CrtPlan &plan, const uint32_t *res32, int64_t nent, int64_t cnt,
                uint64_t *out64, int64_t out_ld, int64_t out_cap, cudaStream_t st)
{
    const int64_t total = nent * out_cap;
    if (total <= 0) return PMLG_OK;
    int64_t blocks = (total + 255) / 256;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    if (blocks > cap) blocks = cap;
    prof_begin(ctx, "crt", st);
    crt_kernel<<<(unsigned)blocks, 256, 0, st>>>(plan, res32, nent, cnt, out64, out_ld, out_cap);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

}  // namespace pmlg
