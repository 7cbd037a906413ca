// approx.cu -- approximant bases: pmbasis divide and conquer on the host
// (approximant_basis.c:33-69), with the middle products and products of
// polymat.cu, and the mbasis leaves on the device (nmod_mat_poly_mbasis.c:116-378).
//
// The leaf kernel runs all order-1 steps of one leaf in one CTA.  It keeps the
// residual R = appbas * F mod x^order (coefficient-major) and updates it with
// the same row operations as appbas, so that the residual of step ord is
// simply R[ord]: coefficient ord of appbas * F is unique, so this gives the
// same steps as recomputing it (nmod_mat_poly_mul_coeff, nmod_mat_poly_arith.c:4-41).
// Each step:
//   1. stable sort of (shift[i], i) (_find_shift_permutation, :99-114);
//   2. Gauss-Jordan elimination of the permuted residual's transpose, giving
//      the row rank profile and the compact left nullspace X = -R[j][np_i]
//      with R the (unique) RREF (left_nullspace.c:42-102); the elimination is
//      division-free (rows are scaled by the pivot instead of divided) and the
//      pivot rows are normalised once at the end, which yields the same RREF;
//   3. the update of appbas and R: non-pivot rows += X * pivot rows, pivot
//      rows multiplied by x, shift of the pivot rows + 1 (:252-359), or, when
//      the nullity is 0, appbas *= x^(order-ord) (:221-231).
#include "polymat.cuh"
#include "ntt.cuh"

#include <vector>

namespace pmlg {

constexpr int LEAF_THREADS = 512;
constexpr int LEAF_MAX = 64;     // m, n <= 64

struct LeafArgs
{
    const uint64_t *F;
    int64_t ldF, flen;
    uint64_t *out;
    int64_t ldo;
    uint32_t *R;      // [order][m][n]
    uint32_t *AB;     // [order+1][m][m]
    int64_t *shift;   // device, m entries
    int m, n, order;
    uint32_t p, r32, r32q, oneq;
};

__device__ __forceinline__ uint32_t mulmod32(uint32_t a, uint32_t b, const LeafArgs &A)
{
    return mod64_q((uint64_t)a * b, A.p, A.r32, A.r32q, A.oneq);
}

__device__ uint32_t invmod32(uint32_t a, const LeafArgs &A)
{
    // Fermat: a^(p-2), p prime
    uint32_t r = 1, b = a;
    uint32_t e = A.p - 2;
    while (e) {
        if (e & 1) r = mulmod32(r, b, A);
        b = mulmod32(b, b, A);
        e >>= 1;
    }
    return r;
}

// acc (< 2^62 + 2^32 after folding) += x*y, folded every 8 terms by the caller
__device__ __forceinline__ uint64_t fold(uint64_t acc, uint32_t r32)
{
    return (acc >> 32) * (uint64_t)r32 + (acc & 0xffffffffull);
}

__global__ void __launch_bounds__(LEAF_THREADS)
mbasis_leaf_kernel(LeafArgs a)
{
    __shared__ uint32_t E[LEAF_MAX][LEAF_MAX + 1];   // transposed permuted residual, n x m
    __shared__ uint32_t X[LEAF_MAX][LEAF_MAX];       // nullity x rank
    __shared__ uint32_t fac[LEAF_MAX], inv[LEAF_MAX];
    __shared__ int perm[LEAF_MAX], pivlane[LEAF_MAX], pivcol[LEAF_MAX], nonpiv[LEAF_MAX];
    __shared__ int pivrow[LEAF_MAX], nprow[LEAF_MAX];
    __shared__ int used[LEAF_MAX];
    __shared__ long long sh[LEAF_MAX];
    __shared__ int s_pl[2], s_rank, s_nn, s_alen, s_grow, s_stop;

    const int tid = threadIdx.x, nth = blockDim.x;
    const int m = a.m, n = a.n, order = a.order;
    const uint32_t p = a.p;
    const int64_t fl = a.flen < order ? a.flen : order;

    for (int64_t idx = tid; idx < (int64_t)order * m * n; idx += nth) {
        const int64_t d = idx / (m * n), rem = idx - d * m * n;
        a.R[idx] = d < fl ? (uint32_t)a.F[rem * a.ldF + d] : 0u;
    }
    for (int64_t idx = tid; idx < (int64_t)(order + 1) * m * m; idx += nth)
        a.AB[idx] = (idx < m * m && (idx / m) == (idx % m)) ? 1u : 0u;
    if (tid < m) sh[tid] = a.shift[tid];
    if (tid == 0) { s_alen = 1; s_stop = 0; }
    __syncthreads();

    for (int ord = 0; ord < order; ord++) {
        // 1. stable sort of (shift, index): rank by counting
        if (tid < m) {
            int r = 0;
            const long long v = sh[tid];
            for (int i = 0; i < m; i++) r += (sh[i] < v) || (sh[i] == v && i < tid);
            perm[r] = tid;
        }
        if (tid < LEAF_MAX) used[tid] = 0;
        if (tid == 0) { s_rank = 0; s_nn = 0; }
        __syncthreads();
        for (int idx = tid; idx < m * n; idx += nth) {
            const int r = idx / n, j = idx - r * n;
            E[j][r] = a.R[((int64_t)ord * m + perm[r]) * n + j];
        }
        __syncthreads();

        // 2. division-free Gauss-Jordan on E (n rows, m columns)
        for (int c = 0; c < m; c++) {
            if (tid < 32) {
                const int l0 = tid, l1 = tid + 32;
                const uint32_t v0 = (l0 < n && !used[l0]) ? E[l0][c] : 0u;
                const uint32_t v1 = (l1 < n && !used[l1]) ? E[l1][c] : 0u;
                const unsigned b0 = __ballot_sync(0xffffffffu, v0 != 0);
                const unsigned b1 = __ballot_sync(0xffffffffu, v1 != 0);
                const int pl = b0 ? __ffs(b0) - 1 : (b1 ? 32 + __ffs(b1) - 1 : -1);
                if (l0 < n) fac[l0] = E[l0][c];
                if (l1 < n) fac[l1] = E[l1][c];
                __syncwarp();
                if (tid == 0) {
                    s_pl[c & 1] = pl;   // double-buffered: slow readers of column c-1 are not overwritten
                    if (pl < 0) {
                        nonpiv[s_nn++] = c;
                    } else {
                        used[pl] = 1;
                        pivlane[s_rank] = pl;
                        pivcol[s_rank] = c;
                        s_rank++;
                    }
                }
            }
            __syncthreads();
            const int pl = s_pl[c & 1];
            if (pl >= 0) {
                const uint32_t pv = E[pl][c];
                for (int idx = tid; idx < n * m; idx += nth) {
                    const int j = idx / m, cc = idx - j * m;
                    if (j == pl) continue;
                    const uint64_t t = (uint64_t)pv * E[j][cc] + (uint64_t)(p - fac[j]) * E[pl][cc];
                    E[j][cc] = mod64_q(t, p, a.r32, a.r32q, a.oneq);
                }
                __syncthreads();
            }
        }
        const int rank = s_rank, nullity = m - rank;
        __syncthreads();   // everyone has read s_rank before it is reset

        if (nullity == 0) {
            // appbas = x^(order-ord) * appbas, shift += order - ord
            const int k = order - ord, alen = s_alen;
            for (int idx = tid; idx < m * m; idx += nth) {
                for (int d = alen - 1; d >= 0; d--) a.AB[(int64_t)(d + k) * m * m + idx] = a.AB[(int64_t)d * m * m + idx];
                for (int d = 0; d < k; d++) a.AB[(int64_t)d * m * m + idx] = 0;
            }
            if (tid < m) sh[tid] += k;
            if (tid == 0) s_alen = alen + k;
            __syncthreads();
            break;
        }
        if (rank == 0) continue;   // zero residual: nothing changes

        // compact nullspace X[a][b] = -E[pl_b][np_a] / E[pl_b][pc_b]
        if (tid < rank) {
            inv[tid] = invmod32(E[pivlane[tid]][pivcol[tid]], a);
            pivrow[tid] = perm[pivcol[tid]];
        }
        if (tid < nullity) nprow[tid] = perm[nonpiv[tid]];
        __syncthreads();
        for (int idx = tid; idx < nullity * rank; idx += nth) {
            const int ia = idx / rank, b = idx - ia * rank;
            const uint32_t v = mulmod32(E[pivlane[b]][nonpiv[ia]], inv[b], a);
            X[ia][b] = v ? p - v : 0u;
        }
        if (tid < rank) sh[pivrow[tid]] += 1;
        if (tid == 0) s_grow = 0;
        __syncthreads();

        // 3a. non-pivot rows += X * pivot rows, for appbas (d < alen) and R (ord < d < order)
        const int alen = s_alen;
        const int64_t nab = (int64_t)nullity * alen * m;
        const int64_t nR = (int64_t)nullity * (order - ord - 1) * n;
        for (int64_t idx = tid; idx < nab + nR; idx += nth) {
            uint32_t *base;
            int row, col, width;
            int64_t coef;
            if (idx < nab) {
                const int ia = (int)(idx / ((int64_t)alen * m));
                const int64_t rem = idx - (int64_t)ia * alen * m;
                coef = rem / m;
                col = (int)(rem - coef * m);
                row = nprow[ia];
                width = m;
                base = a.AB + coef * m * m;
                const uint32_t *src = base;
                uint64_t acc = src[row * width + col];
                int b = 0;
                for (; b + 8 <= rank; b += 8) {
#pragma unroll
                    for (int u = 0; u < 8; u++) acc += (uint64_t)X[ia][b + u] * src[pivrow[b + u] * width + col];
                    acc = fold(acc, a.r32);
                }
                for (; b < rank; b++) acc += (uint64_t)X[ia][b] * src[pivrow[b] * width + col];
                base[row * width + col] = mod64_q(acc, p, a.r32, a.r32q, a.oneq);
            } else {
                const int64_t j2 = idx - nab;
                const int ia = (int)(j2 / ((int64_t)(order - ord - 1) * n));
                const int64_t rem = j2 - (int64_t)ia * (order - ord - 1) * n;
                coef = ord + 1 + rem / n;
                col = (int)(rem % n);
                row = nprow[ia];
                width = n;
                base = a.R + coef * m * n;
                const uint32_t *src = base;
                uint64_t acc = src[row * width + col];
                int b = 0;
                for (; b + 8 <= rank; b += 8) {
#pragma unroll
                    for (int u = 0; u < 8; u++) acc += (uint64_t)X[ia][b + u] * src[pivrow[b + u] * width + col];
                    acc = fold(acc, a.r32);
                }
                for (; b < rank; b++) acc += (uint64_t)X[ia][b] * src[pivrow[b] * width + col];
                base[row * width + col] = mod64_q(acc, p, a.r32, a.r32q, a.oneq);
            }
        }
        // grow test: a pivot row reaches the top coefficient
        for (int idx = tid; idx < rank * m; idx += nth) {
            const int b = idx / m, col = idx - b * m;
            if (a.AB[(int64_t)(alen - 1) * m * m + pivrow[b] * m + col] != 0) s_grow = 1;
        }
        __syncthreads();
        const int nlen = alen + (s_grow ? 1 : 0);
        // 3b. pivot rows *= x, in appbas and in R
        for (int idx = tid; idx < rank * (m + n); idx += nth) {
            const int b = idx / (m + n), col = idx - b * (m + n);
            const int row = pivrow[b];
            if (col < m) {
                for (int d = nlen - 1; d > 0; d--)
                    a.AB[(int64_t)d * m * m + row * m + col] = a.AB[(int64_t)(d - 1) * m * m + row * m + col];
                a.AB[row * m + col] = 0;
            } else {
                const int j = col - m;
                for (int d = order - 1; d > ord; d--)
                    a.R[(int64_t)d * m * n + row * n + j] = a.R[(int64_t)(d - 1) * m * n + row * n + j];
            }
        }
        __syncthreads();
        if (tid == 0) s_alen = nlen;
        __syncthreads();
    }

    // output: entry-major, zero beyond alen
    const int alen = s_alen;
    for (int64_t idx = tid; idx < (int64_t)m * m * a.ldo; idx += nth) {
        const int64_t e = idx / a.ldo, d = idx - e * a.ldo;
        a.out[idx] = d < alen ? (uint64_t)a.AB[d * m * m + e] : 0ull;
    }
    if (tid < m) a.shift[tid] = sh[tid];
}

// ---------------------------------------------------------------------------
// host recursion
// ---------------------------------------------------------------------------

struct Arena
{
    char *base;
    size_t cap, top;
    void *alloc(size_t bytes)
    {
        size_t b = (bytes + 255) & ~(size_t)255;
        if (top + b > cap) return nullptr;
        void *r = base + top;
        top += b;
        return r;
    }
};

// bytes the recursion needs at order o (upper bound)
static size_t pm_arena_bytes(int64_t m, int64_t n, int64_t o, int64_t leaf)
{
    if (o <= leaf) return (size_t)(o * m * n + (o + 1) * m * m) * 4 + 1024;
    const int64_t o1 = o >> 1, o2 = o - o1;
    size_t here = (size_t)(m * m * (o1 + 1) + m * n * o2 + m * m * (o2 + 1)) * 8 + 1024;
    size_t c1 = pm_arena_bytes(m, n, o1, leaf), c2 = pm_arena_bytes(m, n, o2, leaf);
    return here + (c1 > c2 ? c1 : c2);
}

struct PmState
{
    pmlg_ctx *ctx;
    cudaStream_t st;
    Arena ar;
    int64_t m, n, leaf;
    uint64_t p;
    int64_t *d_shift;
    unsigned long long *d_tmp;
};

static int leaf_run(PmState &S, uint64_t *out, int64_t ldo, const uint64_t *F, int64_t ldF, int64_t flen,
                    int64_t order)
{
    const size_t mark = S.ar.top;
    uint32_t *R = (uint32_t *)S.ar.alloc((size_t)(order * S.m * S.n) * 4 + 4);
    uint32_t *AB = (uint32_t *)S.ar.alloc((size_t)((order + 1) * S.m * S.m) * 4);
    if (!R || !AB) return PMLG_ENOMEM;
    LeafArgs a{};
    a.F = F; a.ldF = ldF; a.flen = flen;
    a.out = out; a.ldo = ldo;
    a.R = R; a.AB = AB;
    a.shift = S.d_shift;
    a.m = (int)S.m; a.n = (int)S.n; a.order = (int)order;
    a.p = (uint32_t)S.p;
    a.r32 = (uint32_t)((1ull << 32) % S.p);
    a.r32q = h_shoup_q(a.r32, a.p);
    a.oneq = (uint32_t)((1ull << 32) / S.p);
    prof_begin(S.ctx, "mbasis_leaf", S.st);
    mbasis_leaf_kernel<<<1, LEAF_THREADS, 0, S.st>>>(a);
    prof_end(S.ctx, S.st);
    count_launch(S.ctx);
    pmlg_ctx *ctx = S.ctx;
    PMLG_CUDA_TRY(cudaGetLastError());
    S.ar.top = mark;
    return PMLG_OK;
}

static int run_product(PmState &S, ProductJob &j)
{
    pmlg_ctx *ctx = S.ctx;
    if (j.cnt <= 0) {
        // zero the output window
        for (int64_t e = 0; e < j.r * j.c; e++)
            PMLG_CUDA_TRY(cudaMemsetAsync(j.C + e * j.ldc, 0, (size_t)j.c_cap * 8, S.st));
        return PMLG_OK;
    }
    if (j.lg > kMaxLgN) {
        set_error(ctx, "pmbasis product needs a transform beyond 2^%d", kMaxLgN);
        return PMLG_ELEN;
    }
    CrtPlan plan;
    const int64_t minlen = j.a_len < j.b_len ? j.a_len : j.b_len;
    PMLG_TRY(make_plan(ctx, j.p, j.lg, j.k, minlen, &plan));
    PMLG_TRY(ws_reserve(ctx, &ctx->ws, product_scratch_bytes(j, plan)));
    return product_run(ctx, j, plan, ctx->ws.ptr, ctx->form, S.st);
}

// appbas: m x m, entry stride ldA (>= order + 1); returns its max length in *len
static int pmbasis_rec(PmState &S, uint64_t *appbas, int64_t ldA, const uint64_t *F, int64_t ldF, int64_t flen,
                       int64_t order, int64_t *len)
{
    pmlg_ctx *ctx = S.ctx;
    const int64_t m = S.m, n = S.n;
    const int64_t pl = flen < order ? flen : order;   // set_trunc(F, order)
    if (order <= S.leaf) {
        PMLG_TRY(leaf_run(S, appbas, ldA, F, ldF, pl, order));
        return device_max_length(ctx, appbas, m * m, ldA, ldA, S.d_tmp, len, S.st);
    }
    const int64_t o1 = order >> 1, o2 = order - o1;
    const size_t mark = S.ar.top;
    uint64_t *A1 = (uint64_t *)S.ar.alloc((size_t)(m * m * (o1 + 1)) * 8);
    uint64_t *Res = (uint64_t *)S.ar.alloc((size_t)(m * n * o2) * 8);
    uint64_t *A2 = (uint64_t *)S.ar.alloc((size_t)(m * m * (o2 + 1)) * 8);
    if (!A1 || !Res || !A2) return PMLG_ENOMEM;

    int64_t l1 = 0, l2 = 0;
    PMLG_TRY(pmbasis_rec(S, A1, o1 + 1, F, ldF, pl, o1, &l1));

    // residual = mulmid(appbas, pmat, order1, order)  (approximant_basis.c:60)
    {
        ProductJob j{};
        j.r = m; j.k = m; j.c = n;
        j.A = A1; j.lda = o1 + 1;
        j.B = F; j.ldb = ldF;
        j.C = Res; j.ldc = o2; j.c_cap = o2;
        j.p = S.p;
        mulmid_prepare(j, l1, pl, o1, order);
        PMLG_TRY(run_product(S, j));
    }
    PMLG_TRY(pmbasis_rec(S, A2, o2 + 1, Res, o2, o2, o2, &l2));

    // appbas = appbas2 * appbas  (approximant_basis.c:64)
    {
        ProductJob j{};
        j.r = m; j.k = m; j.c = m;
        j.A = A2; j.lda = o2 + 1; j.a_off = 0; j.a_len = l2;
        j.B = A1; j.ldb = o1 + 1; j.b_off = 0; j.b_len = l1;
        j.C = appbas; j.ldc = ldA; j.c_cap = ldA;
        j.lo = 0;
        j.cnt = (l1 > 0 && l2 > 0) ? l1 + l2 - 1 : 0;
        if (j.cnt > ldA) j.cnt = ldA;
        j.lg = lg_for(j.cnt > 0 ? l1 + l2 - 1 : 1);
        j.p = S.p;
        PMLG_TRY(run_product(S, j));
    }
    S.ar.top = mark;
    return device_max_length(ctx, appbas, m * m, ldA, ldA, S.d_tmp, len, S.st);
}

static int approx_entry(pmlg_ctx *ctx, uint64_t *appbas, int64_t cap, int64_t *shift, const uint64_t *F,
                        int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p, int64_t *out_len,
                        cudaStream_t st, int64_t leaf)
{
    if (!ctx || !shift || m <= 0 || n <= 0 || flen < 0 || order < 0) return PMLG_EINVAL;
    if (cap < order + 1 || !appbas || (flen > 0 && !F)) return PMLG_EINVAL;
    if (m > LEAF_MAX || n > LEAF_MAX) {
        set_error(ctx, "approximant bases support m, n <= %d", LEAF_MAX);
        return PMLG_EUNSUP;
    }
    if (p < 2 || p >= (1ull << 30) || !h_is_prime(p)) {
        set_error(ctx, "approximant bases need a prime p < 2^30");
        return PMLG_EBADMOD;
    }
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t leaf_eff = leaf < 1 ? 1 : leaf;
    const size_t bytes = pm_arena_bytes(m, n, order > 0 ? order : 1, leaf_eff) + (size_t)m * 8 + 1024;
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_pm, bytes));
    PmState S{};
    S.ctx = ctx;
    S.st = st;
    S.ar = Arena{(char *)ctx->ws_pm.ptr, ctx->ws_pm.bytes, 0};
    S.m = m; S.n = n; S.p = p; S.leaf = leaf_eff;
    S.d_shift = (int64_t *)S.ar.alloc((size_t)m * 8);
    S.d_tmp = (unsigned long long *)S.ar.alloc(64);
    PMLG_CUDA_TRY(cudaMemcpyAsync(S.d_shift, shift, (size_t)m * 8, cudaMemcpyHostToDevice, st));
    int64_t len = 0;
    if (order == 0) {
        // identity basis, shift unchanged
        PMLG_CUDA_TRY(cudaMemsetAsync(appbas, 0, (size_t)(m * m * cap) * 8, st));
        std::vector<uint64_t> one(1, 1);
        for (int64_t i = 0; i < m; i++)
            PMLG_CUDA_TRY(cudaMemcpyAsync(appbas + (i * m + i) * cap, one.data(), 8, cudaMemcpyHostToDevice, st));
        len = 1;
    } else {
        PMLG_TRY(pmbasis_rec(S, appbas, cap, F, flen, flen, order, &len));
    }
    PMLG_CUDA_TRY(cudaMemcpyAsync(shift, S.d_shift, (size_t)m * 8, cudaMemcpyDeviceToHost, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    if (out_len) *out_len = len;
    return PMLG_OK;
}

}  // namespace pmlg

using namespace pmlg;

extern "C" {

PMLG_API int pmlg_pmbasis(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                          const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                          uint64_t p, int64_t *appbas_len, void *stream)
{
    if (!ctx) return PMLG_EINVAL;
    const int64_t leaf = ctx->leaf_order > 0 ? ctx->leaf_order : 32;
    return approx_entry(ctx, appbas, appbas_cap, shift, F, m, n, flen, order, p, appbas_len,
                        (cudaStream_t)stream, leaf);
}

PMLG_API int pmlg_mbasis(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                         const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                         uint64_t p, int64_t *appbas_len, void *stream)
{
    return approx_entry(ctx, appbas, appbas_cap, shift, F, m, n, flen, order, p, appbas_len,
                        (cudaStream_t)stream, order > 0 ? order : 1);
}

PMLG_API int pmlg_pmbasis_host(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                               const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                               uint64_t p, int64_t *appbas_len, void *stream)
{
    if (!ctx || m <= 0 || n <= 0 || flen < 0 || appbas_cap < 0) return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const size_t bF = (size_t)(m * n * flen) * 8, bA = (size_t)(m * m * appbas_cap) * 8;
    const size_t oA = (bF + 255) & ~(size_t)255;
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, oA + bA + 256));
    uint64_t *dF = (uint64_t *)ctx->ws_aux.ptr;
    uint64_t *dA = (uint64_t *)((char *)ctx->ws_aux.ptr + oA);
    if (bF) PMLG_CUDA_TRY(cudaMemcpyAsync(dF, F, bF, cudaMemcpyHostToDevice, st));
    PMLG_TRY(pmlg_pmbasis(ctx, dA, appbas_cap, shift, dF, m, n, flen, order, p, appbas_len, stream));
    if (bA) PMLG_CUDA_TRY(cudaMemcpyAsync(appbas, dA, bA, cudaMemcpyDeviceToHost, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    return PMLG_OK;
}

}  // extern "C"
