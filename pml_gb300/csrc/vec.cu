// vec.cu -- modular dot products with delayed reduction, multimodular
// reduction and CRT.
//
// Dot products accumulate the exact integer sum (192-bit per thread for 64-bit
// entries, 128-bit for 32-bit entries), reduce the partial sums across the
// grid exactly, and reduce mod p once at the end: the same delayed-reduction
// idea as nmod_vec_dot_product_unbalanced's 3-limb accumulator
// (flint-extras/src/nmod_vec_extra/nmod_vec_dot_product.c:68-127) and
// _nmod32_vec_dot_split (nmod32_vec/dot_split.c:18-47), without their length
// limits.
#include "pmlg_internal.cuh"

#include <mutex>

namespace pmlg {

struct U192
{
    unsigned long long w0, w1, w2;
};

__device__ __forceinline__ void add128(U192 &a, unsigned long long lo, unsigned long long hi)
{
    // a += hi:lo with carries into w2
    unsigned long long s0 = a.w0 + lo;
    unsigned long long c0 = s0 < lo;
    unsigned long long s1 = a.w1 + hi;
    unsigned long long c1 = s1 < hi;
    unsigned long long s1b = s1 + c0;
    c1 += s1b < c0;
    a.w0 = s0;
    a.w1 = s1b;
    a.w2 += c1;
}

__device__ __forceinline__ void add192(U192 &a, const U192 &b)
{
    add128(a, b.w0, b.w1);
    a.w2 += b.w2;
}

__device__ __forceinline__ U192 shfl_down192(const U192 &v, int o)
{
    U192 r;
    r.w0 = __shfl_down_sync(0xffffffffu, v.w0, o);
    r.w1 = __shfl_down_sync(0xffffffffu, v.w1, o);
    r.w2 = __shfl_down_sync(0xffffffffu, v.w2, o);
    return r;
}

// block-wide exact sum; result valid in thread 0
__device__ U192 block_sum192(U192 v)
{
    __shared__ U192 part[32];
    for (int o = 16; o > 0; o >>= 1) {
        U192 w = shfl_down192(v, o);
        add192(v, w);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) part[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? part[lane] : U192{0, 0, 0};
        for (int o = 16; o > 0; o >>= 1) {
            U192 w = shfl_down192(v, o);
            add192(v, w);
        }
    }
    return v;
}

__device__ __forceinline__ uint64_t mod192(const U192 &v, uint64_t p)
{
    unsigned __int128 acc = v.w2 % p;
    acc = ((acc << 64) | v.w1) % p;
    acc = ((acc << 64) | v.w0) % p;
    return (uint64_t)acc;
}

// Streaming loads: every element is read once, so L1 keeps none of it.
__device__ __forceinline__ ulonglong2 ld_nc2(const ulonglong2 *p)
{
    ulonglong2 v;
    asm("ld.global.nc.L1::no_allocate.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ uint4 ld_nc4(const uint4 *p)
{
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}

__device__ __forceinline__ void mac64(U192 &acc, unsigned long long a, unsigned long long b)
{
    add128(acc, a * b, __umul64hi(a, b));
}

// HBM-bound: with 16-byte vectors of both operands and four of each in flight per
// thread (grid-strided), the loads outstanding cover the latency of the memory system.
constexpr int DOT_UNROLL = 4;

#ifndef PMLG_DOTMULTI_PAIRS
#define PMLG_DOTMULTI_PAIRS 1          // vector-matrix products: two columns per thread
#endif
#ifndef PMLG_DOTMULTI_BLOCKS_PER_SM
#define PMLG_DOTMULTI_BLOCKS_PER_SM 32  // target blocks per SM (row chunks x column blocks)
#endif

__global__ void dot64_partial(const uint64_t *__restrict__ v1, const uint64_t *__restrict__ v2, int64_t len,
                              U192 *part)
{
    U192 acc{0, 0, 0};
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t start = 0;
    if (((reinterpret_cast<uintptr_t>(v1) | reinterpret_cast<uintptr_t>(v2)) & 15) == 0) {
        const ulonglong2 *a2 = reinterpret_cast<const ulonglong2 *>(v1);
        const ulonglong2 *b2 = reinterpret_cast<const ulonglong2 *>(v2);
        const int64_t n2 = len >> 1;
        int64_t i = tid;
        for (; i + (DOT_UNROLL - 1) * stride < n2; i += DOT_UNROLL * stride) {
            ulonglong2 a[DOT_UNROLL], b[DOT_UNROLL];
#pragma unroll
            for (int u = 0; u < DOT_UNROLL; u++) {
                a[u] = ld_nc2(a2 + i + u * stride);
                b[u] = ld_nc2(b2 + i + u * stride);
            }
#pragma unroll
            for (int u = 0; u < DOT_UNROLL; u++) {
                mac64(acc, a[u].x, b[u].x);
                mac64(acc, a[u].y, b[u].y);
            }
        }
        for (; i < n2; i += stride) {
            const ulonglong2 a = ld_nc2(a2 + i), b = ld_nc2(b2 + i);
            mac64(acc, a.x, b.x);
            mac64(acc, a.y, b.y);
        }
        start = n2 << 1;
    }
    for (int64_t i = start + tid; i < len; i += stride) mac64(acc, v1[i], v2[i]);
    acc = block_sum192(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void dot32_partial(const uint32_t *__restrict__ v1, const uint32_t *__restrict__ v2, int64_t len,
                              U192 *part)
{
    // products < 2^64: accumulate in 64 bits and carry into the high words
    U192 acc{0, 0, 0};
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t start = 0;
    if (((reinterpret_cast<uintptr_t>(v1) | reinterpret_cast<uintptr_t>(v2)) & 15) == 0) {
        const uint4 *a4 = reinterpret_cast<const uint4 *>(v1);
        const uint4 *b4 = reinterpret_cast<const uint4 *>(v2);
        const int64_t n4 = len >> 2;
        int64_t i = tid;
        for (; i + (DOT_UNROLL - 1) * stride < n4; i += DOT_UNROLL * stride) {
            uint4 a[DOT_UNROLL], b[DOT_UNROLL];
#pragma unroll
            for (int u = 0; u < DOT_UNROLL; u++) {
                a[u] = ld_nc4(a4 + i + u * stride);
                b[u] = ld_nc4(b4 + i + u * stride);
            }
#pragma unroll
            for (int u = 0; u < DOT_UNROLL; u++) {
                add128(acc, (uint64_t)a[u].x * b[u].x, 0);
                add128(acc, (uint64_t)a[u].y * b[u].y, 0);
                add128(acc, (uint64_t)a[u].z * b[u].z, 0);
                add128(acc, (uint64_t)a[u].w * b[u].w, 0);
            }
        }
        for (; i < n4; i += stride) {
            const uint4 a = ld_nc4(a4 + i), b = ld_nc4(b4 + i);
            add128(acc, (uint64_t)a.x * b.x, 0);
            add128(acc, (uint64_t)a.y * b.y, 0);
            add128(acc, (uint64_t)a.z * b.z, 0);
            add128(acc, (uint64_t)a.w * b.w, 0);
        }
        start = n4 << 2;
    }
    for (int64_t i = start + tid; i < len; i += stride) add128(acc, (uint64_t)v1[i] * v2[i], 0);
    acc = block_sum192(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void dot_final(const U192 *part, int nparts, uint64_t p, uint64_t *res64, uint32_t *res32)
{
    U192 acc{0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) add192(acc, part[i]);
    acc = block_sum192(acc);
    if (threadIdx.x == 0) {
        const uint64_t r = mod192(acc, p);
        if (res64) *res64 = r;
        if (res32) *res32 = (uint32_t)r;
    }
}

// one warp per row: mv[i] = sum_j mat[i*stride + j] * vec[j] mod p
__global__ void mdot32_kernel(uint32_t *mv, const uint32_t *__restrict__ mat, const uint32_t *__restrict__ vec,
                              int64_t nrows, int64_t len, int64_t stride, uint64_t p)
{
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    const uint32_t *row = mat + warp * stride;
    U192 acc{0, 0, 0};
    for (int64_t j = lane; j < len; j += 32) add128(acc, (uint64_t)row[j] * vec[j], 0);
    for (int o = 16; o > 0; o >>= 1) {
        U192 w = shfl_down192(acc, o);
        add192(acc, w);
    }
    if (lane == 0) mv[warp] = (uint32_t)mod192(acc, p);
}

// one 256-thread block per row, for rows of at least 4096 entries: sixteen times
// more (and shorter) tasks than rows of one warp, so the last wave of a tall matrix
// leaves few SMs idle
constexpr int MDOT_BLOCK = 256;
__global__ void __launch_bounds__(MDOT_BLOCK)
mdot32_block_kernel(uint32_t *mv, const uint32_t *__restrict__ mat, const uint32_t *__restrict__ vec,
                    int64_t len, int64_t stride, uint64_t p)
{
    const uint32_t *row = mat + (int64_t)blockIdx.x * stride;
    U192 acc{0, 0, 0};
    for (int64_t j = threadIdx.x; j < len; j += MDOT_BLOCK) add128(acc, (uint64_t)row[j] * vec[j], 0);
    acc = block_sum192(acc);
    if (threadIdx.x == 0) mv[blockIdx.x] = (uint32_t)mod192(acc, p);
}

// uv[j] = sum_i u[i] * v[i*k + j]: grid.x over columns, grid.y over chunks of i; eight
// rows of v in flight per thread
__global__ void dot_multi_partial(const uint64_t *__restrict__ u, const uint64_t *__restrict__ v, int64_t len,
                                  int64_t k, int64_t chunk, U192 *part)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k) return;
    const int64_t i0 = (int64_t)blockIdx.y * chunk;
    const int64_t i1 = i0 + chunk < len ? i0 + chunk : len;
    U192 acc{0, 0, 0};
    int64_t i = i0;
    for (; i + 8 <= i1; i += 8) {
        uint64_t a[8], b[8];
#pragma unroll
        for (int t = 0; t < 8; t++) {
            a[t] = __ldg(u + i + t);
            b[t] = v[(i + t) * k + j];
        }
#pragma unroll
        for (int t = 0; t < 8; t++) mac64(acc, a[t], b[t]);
    }
    for (; i < i1; i++) mac64(acc, u[i], v[i * k + j]);
    part[(int64_t)blockIdx.y * k + j] = acc;
}

// the same, two adjacent columns per thread (k even, v 16-byte aligned): 16-byte loads,
// four rows in flight
__global__ void dot_multi_partial2(const uint64_t *__restrict__ u, const uint64_t *__restrict__ v, int64_t len,
                                   int64_t k, int64_t chunk, U192 *part)
{
    const int64_t j2 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;   // column pair
    if (2 * j2 >= k) return;
    const int64_t i0 = (int64_t)blockIdx.y * chunk;
    const int64_t i1 = i0 + chunk < len ? i0 + chunk : len;
    const ulonglong2 *v2 = reinterpret_cast<const ulonglong2 *>(v);
    const int64_t k2 = k >> 1;
    U192 acc0{0, 0, 0}, acc1{0, 0, 0};
    int64_t i = i0;
    for (; i + 4 <= i1; i += 4) {
        uint64_t a[4];
        ulonglong2 b[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            a[t] = __ldg(u + i + t);
            b[t] = ld_nc2(v2 + (i + t) * k2 + j2);
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            mac64(acc0, a[t], b[t].x);
            mac64(acc1, a[t], b[t].y);
        }
    }
    for (; i < i1; i++) {
        const ulonglong2 b = ld_nc2(v2 + i * k2 + j2);
        mac64(acc0, u[i], b.x);
        mac64(acc1, u[i], b.y);
    }
    part[(int64_t)blockIdx.y * k + 2 * j2] = acc0;
    part[(int64_t)blockIdx.y * k + 2 * j2 + 1] = acc1;
}

__global__ void dot_multi_final(const U192 *part, int64_t nchunks, int64_t k, uint64_t p, uint64_t *uv)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k) return;
    U192 acc{0, 0, 0};
    for (int64_t c = 0; c < nchunks; c++) add192(acc, part[c * k + j]);
    uv[j] = mod192(acc, p);
}

// residues[j*nb + i] = x[i] mod q_j; Barrett quotient estimate with m_j = floor((2^64-1)/q_j)
struct MultimodArgs
{
    int t;
    uint64_t q[kMaxPrimes], m[kMaxPrimes];
};

__global__ void multimod_reduce_kernel(uint64_t *res, const uint64_t *__restrict__ x, int64_t nb, MultimodArgs a)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t v = x[i];
        for (int j = 0; j < a.t; j++) {
            const uint64_t qe = __umul64hi(v, a.m[j]);
            uint64_t r = v - qe * a.q[j];
            while (r >= a.q[j]) r -= a.q[j];
            res[j * nb + i] = r;
        }
    }
}

struct CrtArgs64
{
    int t;
    uint64_t q[kMaxPrimes];
    uint64_t ginv[kMaxPrimes];         // (q_0 ... q_{j-1})^{-1} mod q_j
    uint64_t p;
};

__device__ __forceinline__ uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m)
{
    return (uint64_t)(((unsigned __int128)a * b) % m);
}

__global__ void multimod_crt_kernel(uint64_t *out, const uint64_t *__restrict__ res, int64_t nb, CrtArgs64 a)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t c[kMaxPrimes];
        for (int j = 0; j < a.t; j++) {
            const uint64_t qj = a.q[j];
            uint64_t v = 0;
            for (int l = j - 1; l >= 0; l--) v = (mulmod64(v, a.q[l] % qj, qj) + c[l] % qj) % qj;
            const uint64_t r = res[j * nb + i] % qj;
            const uint64_t d = r >= v ? r - v : r + (qj - v);
            c[j] = (j == 0) ? r : mulmod64(d, a.ginv[j], qj);
        }
        uint64_t x = 0;
        for (int l = a.t - 1; l >= 0; l--) {
            unsigned __int128 y = (unsigned __int128)x * (a.q[l] % a.p) + (c[l] % a.p);
            x = (uint64_t)(y % a.p);
        }
        out[i] = x;
    }
}

// The same Garner CRT and Horner evaluation without 128-bit division, for p < 2^63
// (the primes are below 2^63 already): any 64-bit value is reduced by a Barrett step
// with mq = floor((2^64-1)/q), which leaves at most two subtractions, and every product
// by a fixed factor w < q is a 64-bit Shoup product with ws = floor(w 2^64 / q), exact
// for any 64-bit multiplicand and q < 2^63.  All factors and quotients come from the host.
struct CrtArgs64Fast
{
    int t;
    uint64_t q[kMaxPrimes], mq[kMaxPrimes];
    uint64_t qlj[kMaxPrimes][kMaxPrimes], qljs[kMaxPrimes][kMaxPrimes];   // q_l mod q_j, l < j
    uint64_t ginv[kMaxPrimes], ginvs[kMaxPrimes];
    uint64_t p, mp;
    uint64_t qlp[kMaxPrimes], qlps[kMaxPrimes];                           // q_l mod p
};

__device__ __forceinline__ uint64_t red64(uint64_t v, uint64_t q, uint64_t mq)
{
    uint64_t r = v - __umul64hi(v, mq) * q;
    r = r >= q ? r - q : r;
    return r >= q ? r - q : r;
}

__device__ __forceinline__ uint64_t shoup64(uint64_t v, uint64_t w, uint64_t ws, uint64_t q)
{
    const uint64_t r = v * w - __umul64hi(v, ws) * q;   // in [0, 2q)
    return r >= q ? r - q : r;
}

// T primes, a compile-time count: the digits c[] stay in registers
template <int T>
__global__ void multimod_crt_fast_kernel(uint64_t *out, const uint64_t *__restrict__ res, int64_t nb,
                                         CrtArgs64Fast a)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t c[T];
        c[0] = red64(res[i], a.q[0], a.mq[0]);
#pragma unroll
        for (int j = 1; j < T; j++) {
            const uint64_t qj = a.q[j], mj = a.mq[j];
            // c_0 + c_1 q_0 + ... + c_{j-1} q_0 ... q_{j-2} mod q_j, by Horner from the top
            uint64_t v = red64(c[j - 1], qj, mj);
#pragma unroll
            for (int l = j - 2; l >= 0; l--) {
                v = shoup64(v, a.qlj[l][j], a.qljs[l][j], qj) + red64(c[l], qj, mj);
                v = v >= qj ? v - qj : v;
            }
            const uint64_t r = red64(res[j * nb + i], qj, mj);
            const uint64_t d = r >= v ? r - v : r + (qj - v);
            c[j] = shoup64(d, a.ginv[j], a.ginvs[j], qj);
        }
        uint64_t x = red64(c[T - 1], a.p, a.mp);
#pragma unroll
        for (int l = T - 2; l >= 0; l--) {
            x = shoup64(x, a.qlp[l], a.qlps[l], a.p) + red64(c[l], a.p, a.mp);
            x = x >= a.p ? x - a.p : x;
        }
        out[i] = x;
    }
}

static int grid_for(pmlg_ctx *ctx, int64_t n, int threads, int per_sm)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)ctx->sm_count * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace pmlg

using namespace pmlg;

extern "C" {

PMLG_API int pmlg_nmod_vec_dot(pmlg_ctx *ctx, uint64_t *res, const uint64_t *v1, const uint64_t *v2,
                               int64_t len, uint64_t p, void *stream)
{
    if (!ctx || !res || len < 0 || (len > 0 && (!v1 || !v2))) return PMLG_EINVAL;
    if (p < 2) return PMLG_EBADMOD;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int threads = 256;
    const int blocks = grid_for(ctx, len, threads, 4);
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, sizeof(U192) * (size_t)blocks + 256));
    U192 *part = (U192 *)ctx->ws_aux.ptr;
    prof_begin(ctx, "dot64_partial", st);
    dot64_partial<<<blocks, threads, 0, st>>>(v1, v2, len, part);
    prof_end(ctx, st);
    prof_begin(ctx, "dot_final", st);
    dot_final<<<1, 256, 0, st>>>(part, blocks, p, res, nullptr);
    prof_end(ctx, st);
    count_launch(ctx, 2);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

PMLG_API int pmlg_nmod32_vec_dot(pmlg_ctx *ctx, uint32_t *res, const uint32_t *v1, const uint32_t *v2,
                                 int64_t len, uint64_t p, void *stream)
{
    if (!ctx || !res || len < 0 || (len > 0 && (!v1 || !v2))) return PMLG_EINVAL;
    if (p < 2 || p > (1ull << 32)) return PMLG_EBADMOD;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int threads = 256;
    const int blocks = grid_for(ctx, (len + 3) / 4, threads, 4);
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, sizeof(U192) * (size_t)blocks + 256));
    U192 *part = (U192 *)ctx->ws_aux.ptr;
    prof_begin(ctx, "dot32_partial", st);
    dot32_partial<<<blocks, threads, 0, st>>>(v1, v2, len, part);
    prof_end(ctx, st);
    prof_begin(ctx, "dot_final", st);
    dot_final<<<1, 256, 0, st>>>(part, blocks, p, nullptr, res);
    prof_end(ctx, st);
    count_launch(ctx, 2);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

PMLG_API int pmlg_nmod32_vec_mdot(pmlg_ctx *ctx, uint32_t *mv, const uint32_t *mat, const uint32_t *vec,
                                  int64_t nrows, int64_t len, int64_t stride, uint64_t p, void *stream)
{
    if (!ctx || nrows < 0 || len < 0 || stride < len) return PMLG_EINVAL;
    if (nrows == 0) return PMLG_OK;
    if (!mv || (len > 0 && (!mat || !vec))) return PMLG_EINVAL;
    if (p < 2 || p > (1ull << 32)) return PMLG_EBADMOD;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    prof_begin(ctx, "mdot32", st);
    if (len >= 4096 && nrows <= 0x7fffffffll) {
        mdot32_block_kernel<<<(unsigned)nrows, MDOT_BLOCK, 0, st>>>(mv, mat, vec, len, stride, p);
    } else {
        const int threads = 256;
        const int64_t blocks = (nrows * 32 + threads - 1) / threads;
        mdot32_kernel<<<(unsigned)blocks, threads, 0, st>>>(mv, mat, vec, nrows, len, stride, p);
    }
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

PMLG_API int pmlg_nmod_vec_dot_multi(pmlg_ctx *ctx, uint64_t *uv, const uint64_t *u, const uint64_t *v,
                                     int64_t len, int64_t k, uint64_t p, void *stream)
{
    if (!ctx || len < 0 || k < 0) return PMLG_EINVAL;
    if (k == 0) return PMLG_OK;
    if (!uv || (len > 0 && (!u || !v))) return PMLG_EINVAL;
    if (p < 2) return PMLG_EBADMOD;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int threads = 128;
    const bool pairs = PMLG_DOTMULTI_PAIRS && (k & 1) == 0 && (reinterpret_cast<uintptr_t>(v) & 15) == 0;
    const int64_t gx = ((pairs ? k / 2 : k) + threads - 1) / threads;
    // enough chunks along i to fill the GPU, each at least 64 rows long
    int64_t nchunks = ((int64_t)ctx->sm_count * PMLG_DOTMULTI_BLOCKS_PER_SM + gx - 1) / gx;
    if (nchunks > (len + 63) / 64) nchunks = (len + 63) / 64;
    if (nchunks < 1) nchunks = 1;
    if (nchunks > 65535) nchunks = 65535;
    const int64_t chunk = (len + nchunks - 1) / nchunks > 0 ? (len + nchunks - 1) / nchunks : 1;
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, sizeof(U192) * (size_t)(nchunks * k) + 256));
    U192 *part = (U192 *)ctx->ws_aux.ptr;
    prof_begin(ctx, "dot_multi_partial", st);
    if (pairs)
        dot_multi_partial2<<<dim3((unsigned)gx, (unsigned)nchunks), threads, 0, st>>>(u, v, len, k, chunk, part);
    else
        dot_multi_partial<<<dim3((unsigned)gx, (unsigned)nchunks), threads, 0, st>>>(u, v, len, k, chunk, part);
    prof_end(ctx, st);
    prof_begin(ctx, "dot_multi_final", st);
    dot_multi_final<<<(unsigned)((k + threads - 1) / threads), threads, 0, st>>>(part, nchunks, k, p, uv);
    prof_end(ctx, st);
    count_launch(ctx, 2);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Vector-matrix dot product without any allocation
// ---------------------------------------------------------------------------
//
// Same kernels as pmlg_nmod_vec_dot_multi, but the partial sums live in a
// file-scope device array instead of context scratch, so the call needs no
// pmlg_ctx and never calls cudaMalloc/cudaFree.  The array is part of the
// library's device image: every GPU that loads the library holds its
// kNoAllocPartials * 24 bytes (1.5 MiB) until the process exits.

namespace pmlg {

constexpr int64_t kNoAllocPartials = 65536;   // largest number of columns k
static __device__ __align__(256) U192 g_noalloc_partials[kNoAllocPartials];

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static U192 *g_noalloc_ptr[kNoAllocMaxDevices];   // device address of the array, per device
static int g_noalloc_sms[kNoAllocMaxDevices];

}  // namespace pmlg

extern "C" {

PMLG_API int pmlg_nmod_vec_dot_multi_noalloc(uint64_t *uv, const uint64_t *u, const uint64_t *v, int64_t len,
                                             int64_t k, uint64_t p, void *stream)
{
    if (len < 0 || k < 0) return PMLG_EINVAL;
    if (k == 0) return PMLG_OK;
    if (!uv || (len > 0 && (!u || !v))) return PMLG_EINVAL;
    if (p < 2) return PMLG_EBADMOD;
    if (k > kNoAllocPartials) return PMLG_EUNSUP;   // the fixed scratch holds at most this many columns
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PMLG_ECUDA;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return PMLG_EUNSUP;
    U192 *part = nullptr;
    int sms = 0;
    {
        // first call on this device: resolve the array's device address with the
        // device current (host code cannot use the symbol itself as a pointer)
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            void *addr = nullptr;
            if (cudaGetSymbolAddress(&addr, g_noalloc_partials) != cudaSuccess || !addr) return PMLG_ECUDA;
            int n = 0;
            if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PMLG_ECUDA;
            g_noalloc_sms[dev] = n;
            g_noalloc_ptr[dev] = (U192 *)addr;
        }
        part = g_noalloc_ptr[dev];
        sms = g_noalloc_sms[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int threads = 128;
    const int64_t gx = (k + threads - 1) / threads;
    int64_t nchunks = ((int64_t)sms * 8 + gx - 1) / gx;
    if (nchunks > (len + 63) / 64) nchunks = (len + 63) / 64;
    if (nchunks > kNoAllocPartials / k) nchunks = kNoAllocPartials / k;   // nchunks * k partials fit
    if (nchunks > 65535) nchunks = 65535;
    if (nchunks < 1) nchunks = 1;
    const int64_t chunk = (len + nchunks - 1) / nchunks > 0 ? (len + nchunks - 1) / nchunks : 1;
    // every partial that dot_multi_final reads is written by dot_multi_partial in
    // this same call, so nothing left in the array by an earlier call is used
    dot_multi_partial<<<dim3((unsigned)gx, (unsigned)nchunks), threads, 0, st>>>(u, v, len, k, chunk, part);
    dot_multi_final<<<(unsigned)gx, threads, 0, st>>>(part, nchunks, k, p, uv);
    if (cudaGetLastError() != cudaSuccess) return PMLG_ECUDA;
    return PMLG_OK;
}

PMLG_API int pmlg_multimod_reduce(pmlg_ctx *ctx, uint64_t *residues, const uint64_t *input, int64_t nb,
                                  const uint64_t *primes, int nprimes, void *stream)
{
    if (!ctx || nb < 0 || !primes || nprimes < 1 || nprimes > kMaxPrimes) return PMLG_EINVAL;
    if (nb == 0) return PMLG_OK;
    if (!residues || !input) return PMLG_EINVAL;
    MultimodArgs a{};
    a.t = nprimes;
    for (int j = 0; j < nprimes; j++) {
        if (primes[j] < 2 || primes[j] >= (1ull << 63)) return PMLG_EBADMOD;
        a.q[j] = primes[j];
        a.m[j] = ~0ull / primes[j];
    }
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    prof_begin(ctx, "multimod_reduce", st);
    multimod_reduce_kernel<<<grid_for(ctx, nb, 256, 8), 256, 0, st>>>(residues, input, nb, a);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

PMLG_API int pmlg_multimod_crt(pmlg_ctx *ctx, uint64_t *out, const uint64_t *residues, int64_t nb,
                               const uint64_t *primes, int nprimes, uint64_t p, void *stream)
{
    if (!ctx || nb < 0 || !primes || nprimes < 1 || nprimes > kMaxPrimes) return PMLG_EINVAL;
    if (p < 2) return PMLG_EBADMOD;
    if (nb == 0) return PMLG_OK;
    if (!out || !residues) return PMLG_EINVAL;
    CrtArgs64 a{};
    a.t = nprimes;
    a.p = p;
    for (int j = 0; j < nprimes; j++) {
        if (primes[j] < 2 || primes[j] >= (1ull << 63)) return PMLG_EBADMOD;
        a.q[j] = primes[j];
        uint64_t pr = 1 % primes[j];
        for (int l = 0; l < j; l++) pr = h_mulmod(pr, primes[l] % primes[j], primes[j]);
        a.ginv[j] = (j == 0) ? 1 : h_invmod(pr, primes[j]);
        if (j > 0 && a.ginv[j] == 0) {
            set_error(ctx, "CRT primes are not pairwise coprime");
            return PMLG_EBADMOD;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    prof_begin(ctx, "multimod_crt", st);
    if (p < (1ull << 63)) {
        auto shoup_q = [](uint64_t w, uint64_t q) { return (uint64_t)(((unsigned __int128)w << 64) / q); };
        CrtArgs64Fast f{};
        f.t = nprimes;
        f.p = p;
        f.mp = ~0ull / p;
        for (int j = 0; j < nprimes; j++) {
            const uint64_t qj = primes[j];
            f.q[j] = qj;
            f.mq[j] = ~0ull / qj;
            f.ginv[j] = a.ginv[j] % qj;
            f.ginvs[j] = shoup_q(f.ginv[j], qj);
            for (int l = 0; l < j; l++) {
                f.qlj[l][j] = primes[l] % qj;
                f.qljs[l][j] = shoup_q(f.qlj[l][j], qj);
            }
            f.qlp[j] = qj % p;
            f.qlps[j] = shoup_q(f.qlp[j], p);
        }
        const int g = grid_for(ctx, nb, 256, 8);
        switch (nprimes) {
        case 1: multimod_crt_fast_kernel<1><<<g, 256, 0, st>>>(out, residues, nb, f); break;
        case 2: multimod_crt_fast_kernel<2><<<g, 256, 0, st>>>(out, residues, nb, f); break;
        case 3: multimod_crt_fast_kernel<3><<<g, 256, 0, st>>>(out, residues, nb, f); break;
        case 4: multimod_crt_fast_kernel<4><<<g, 256, 0, st>>>(out, residues, nb, f); break;
        case 5: multimod_crt_fast_kernel<5><<<g, 256, 0, st>>>(out, residues, nb, f); break;
        default: multimod_crt_fast_kernel<6><<<g, 256, 0, st>>>(out, residues, nb, f); break;
        }
    } else {
        multimod_crt_kernel<<<grid_for(ctx, nb, 256, 8), 256, 0, st>>>(out, residues, nb, a);
    }
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

}  // extern "C"
