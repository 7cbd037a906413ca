// kernel.cu -- left kernel bases of polynomial matrices over Z/pZ:
// nmod_poly_mat_kernel_zls_approx (flint-extras/src/nmod_poly_mat_extra/kernel.c:232-480),
// the Zhou-Labahn-Storjohann recursion through approximant bases.
//
// The recursion itself is host C++ (it branches on degrees and ranks), every
// polynomial matrix lives in device memory, and the arithmetic is the library's:
// pmbasis (approx.cu), products and middle products (polymat.cu).  The host reads
// only entry lengths (one small reduction kernel per decision) and the shifts that
// pmbasis returns.  Each step follows kernel.c line by line, so the output equals
// the reference's for the same pmbasis and products, which are exact.
#include "pmlg_internal.cuh"
#include "leaf64.cuh"
#include "polymat.cuh"

#include <algorithm>
#include <vector>

namespace pmlg {

// length (index of the last nonzero coefficient + 1) of every entry: one block per entry
__global__ void entry_lengths_kernel(const uint64_t *__restrict__ P, int64_t cap, int *__restrict__ out)
{
    const uint64_t *e = P + (int64_t)blockIdx.x * cap;
    int best = 0;
    for (int64_t d = threadIdx.x; d < cap; d += blockDim.x)
        if (e[d] != 0) best = (int)d + 1;
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_down_sync(0xffffffffu, best, o));
    __shared__ int part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = max(best, part[w]);
        out[blockIdx.x] = best;
    }
}

int entry_lengths(pmlg_ctx *ctx, const uint64_t *P, int64_t nent, int64_t cap, int *d_out, std::vector<int> &len,
                  cudaStream_t st)
{
    len.assign((size_t)nent, 0);
    if (nent == 0) return PMLG_OK;
    prof_begin(ctx, "entry_lengths", st);
    entry_lengths_kernel<<<(unsigned)nent, 128, 0, st>>>(P, cap, d_out);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    PMLG_CUDA_TRY(cudaMemcpyAsync(len.data(), d_out, (size_t)nent * sizeof(int), cudaMemcpyDeviceToHost, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    return PMLG_OK;
}

namespace {

// a polynomial matrix in device memory: entry (i, j) at a + (i * c + j) * cap
struct DevPm
{
    uint64_t *a = nullptr;
    int64_t r = 0, c = 0, cap = 1;
};

class Kzls
{
  public:
    Kzls(pmlg_ctx *c, uint64_t p, cudaStream_t st) : ctx(c), p_(p), st_(st) {}
    ~Kzls()
    {
        if (d_len_) cudaFreeAsync(d_len_, st_);
    }

    int alloc(DevPm &P, int64_t r, int64_t c, int64_t cap)
    {
        P.r = r; P.c = c; P.cap = cap > 0 ? cap : 1;
        const size_t bytes = (size_t)(r * c * P.cap) * 8 + 8;
        PMLG_CUDA_TRY(cudaMallocAsync((void **)&P.a, bytes, st_));
        PMLG_CUDA_TRY(cudaMemsetAsync(P.a, 0, bytes, st_));
        return PMLG_OK;
    }
    void release(DevPm &P)
    {
        if (P.a) cudaFreeAsync(P.a, st_);
        P.a = nullptr;
    }

    // lengths of all entries, row-major (synchronises the stream)
    int lengths(const DevPm &P, std::vector<int> &len)
    {
        const int64_t ne = P.r * P.c;
        len.assign((size_t)ne, 0);
        if (ne == 0) return PMLG_OK;
        if (ne > len_cap_) {
            if (d_len_) PMLG_CUDA_TRY(cudaFreeAsync(d_len_, st_));
            PMLG_CUDA_TRY(cudaMallocAsync((void **)&d_len_, (size_t)ne * sizeof(int), st_));
            len_cap_ = ne;
        }
        return entry_lengths(ctx, P.a, ne, P.cap, d_len_, len, st_);
    }
    int max_length(const DevPm &P, int64_t *L)
    {
        std::vector<int> len;
        PMLG_TRY(lengths(P, len));
        int m = 0;
        for (int v : len) m = std::max(m, v);
        *L = m;
        return PMLG_OK;
    }

    // rows [r0, r1), columns [c0, c1), capacity cap (coefficients past P.cap are zero)
    int window(const DevPm &P, int64_t r0, int64_t r1, int64_t c0, int64_t c1, int64_t cap, DevPm &Q)
    {
        PMLG_TRY(alloc(Q, r1 - r0, c1 - c0, cap));
        const int64_t w = std::min(cap, P.cap);
        if (Q.r == 0 || Q.c == 0 || w <= 0) return PMLG_OK;
        // one 2-D copy: rows = entries of the window, width = w coefficients
        for (int64_t i = r0; i < r1; i++)
            PMLG_CUDA_TRY(cudaMemcpy2DAsync(Q.a + (i - r0) * Q.c * Q.cap, (size_t)Q.cap * 8,
                                            P.a + (i * P.c + c0) * P.cap, (size_t)P.cap * 8, (size_t)w * 8,
                                            (size_t)Q.c, cudaMemcpyDeviceToDevice, st_));
        return PMLG_OK;
    }

    // A * B with both trimmed to their exact lengths (nmod_poly_mat_multiply)
    int mul(const DevPm &A, const DevPm &B, DevPm &C)
    {
        int64_t la = 0, lb = 0;
        PMLG_TRY(max_length(A, &la));
        PMLG_TRY(max_length(B, &lb));
        if (la == 0 || lb == 0) return alloc(C, A.r, B.c, 1);
        DevPm At, Bt;
        PMLG_TRY(window(A, 0, A.r, 0, A.c, la, At));
        PMLG_TRY(window(B, 0, B.r, 0, B.c, lb, Bt));
        PMLG_TRY(alloc(C, A.r, B.c, la + lb - 1));
        const int s = poly_mat_mul_device(ctx, C.a, At.a, Bt.a, A.r, A.c, B.c, la, lb, p_, st_);
        release(At);
        release(Bt);
        return s;
    }

    // rows[i] <- rows[perm[i]] for i < nrows
    int permute_rows(DevPm &P, int64_t nrows, const int64_t *perm)
    {
        if (nrows <= 0) return PMLG_OK;
        DevPm T;
        PMLG_TRY(alloc(T, nrows, P.c, P.cap));
        const size_t row = (size_t)(P.c * P.cap) * 8;
        for (int64_t i = 0; i < nrows; i++)
            PMLG_CUDA_TRY(cudaMemcpyAsync((char *)T.a + i * row, (char *)P.a + perm[i] * row, row,
                                          cudaMemcpyDeviceToDevice, st_));
        PMLG_CUDA_TRY(cudaMemcpyAsync(P.a, T.a, row * nrows, cudaMemcpyDeviceToDevice, st_));
        release(T);
        return PMLG_OK;
    }

    // rows [dst0, dst0 + Q.r) of P <- rows of Q (same columns); P's capacity grows if needed
    int set_rows(DevPm &P, int64_t dst0, const DevPm &Q)
    {
        if (Q.cap > P.cap) {
            DevPm W;
            PMLG_TRY(window(P, 0, P.r, 0, P.c, Q.cap, W));
            release(P);
            P = W;
        }
        PMLG_CUDA_TRY(cudaMemsetAsync(P.a + dst0 * P.c * P.cap, 0, (size_t)(Q.r * P.c * P.cap) * 8, st_));
        if (Q.r > 0)
            PMLG_CUDA_TRY(cudaMemcpy2DAsync(P.a + dst0 * P.c * P.cap, (size_t)P.cap * 8, Q.a, (size_t)Q.cap * 8,
                                            (size_t)Q.cap * 8, (size_t)(Q.r * Q.c), cudaMemcpyDeviceToDevice,
                                            st_));
        return PMLG_OK;
    }

    int identity(DevPm &K, int64_t m)
    {
        PMLG_TRY(alloc(K, m, m, 1));
        const uint64_t one = 1;
        for (int64_t i = 0; i < m; i++)
            PMLG_CUDA_TRY(cudaMemcpyAsync(K.a + (i * m + i), &one, 8, cudaMemcpyHostToDevice, st_));
        PMLG_CUDA_TRY(cudaStreamSynchronize(st_));   // `one` lives on this stack frame
        return PMLG_OK;
    }

    // nmod_poly_mat_kernel_zls_approx (kernel.c:232-480); K receives an m x m
    // matrix whose rows [0, *nullity) are the kernel basis
    int run(DevPm &K, int64_t *pivind, int64_t *shift, const DevPm &pm, int64_t *nullity_out);

  private:
    pmlg_ctx *ctx;
    uint64_t p_;
    cudaStream_t st_;
    int *d_len_ = nullptr;
    int64_t len_cap_ = 0;
};

int Kzls::run(DevPm &K, int64_t *pivind, int64_t *shift, const DevPm &pm, int64_t *nullity_out)
{
    const int64_t m = pm.r, n = pm.c;
    std::vector<int> len;
    if (m > 0 && n > 0) PMLG_TRY(lengths(pm, len));
    const int plen = len.empty() ? 0 : *std::max_element(len.begin(), len.end());

    // empty matrices, or single row/column vectors that are zero (:240-248)
    if (m == 0 || n == 0 || ((m == 1 || n == 1) && plen == 0)) {
        PMLG_TRY(identity(K, m));
        for (int64_t i = 0; i < m; i++) pivind[i] = i;
        *nullity_out = m;
        return PMLG_OK;
    }
    // one nonzero row (:251-252)
    if (m == 1) {
        PMLG_TRY(alloc(K, m, m, 1));
        *nullity_out = 0;
        return PMLG_OK;
    }

    // 2n > m: split the columns [n - n/2 | n/2] (:256-317)
    if (2 * n > m) {
        const int64_t n1 = n - n / 2;
        DevPm left;
        PMLG_TRY(window(pm, 0, m, 0, n1, pm.cap, left));
        int64_t nullity = 0;
        const int s1 = run(K, pivind, shift, left, &nullity);
        release(left);
        PMLG_TRY(s1);
        if (nullity == 0) {
            *nullity_out = 0;
            return PMLG_OK;
        }
        DevPm ker1, right, resid, k2;
        PMLG_TRY(window(K, 0, nullity, 0, m, K.cap, ker1));
        PMLG_TRY(window(pm, 0, m, n1, n, pm.cap, right));
        PMLG_TRY(mul(ker1, right, resid));
        release(right);
        std::vector<int64_t> piv2((size_t)nullity);
        int64_t nullity2 = 0;
        const int s2 = run(k2, piv2.data(), shift, resid, &nullity2);
        release(resid);
        if (s2 != PMLG_OK) {
            release(ker1);
            release(k2);
            return s2;
        }
        if (nullity2 > 0) {
            DevPm k2top, k3;
            PMLG_TRY(window(k2, 0, nullity2, 0, nullity, k2.cap, k2top));
            PMLG_TRY(mul(k2top, ker1, k3));
            PMLG_TRY(set_rows(K, 0, k3));
            for (int64_t i = 0; i < nullity2; i++) pivind[i] = pivind[piv2[i]];
            release(k2top);
            release(k3);
        }
        release(k2);
        release(ker1);
        *nullity_out = nullity2;
        return PMLG_OK;
    }

    // 1 <= n <= m/2 (:321-479): max(0, rdeg(pmat)) and the number of nonzero rows
    std::vector<int64_t> buf((size_t)m);
    int64_t nnz = 0;
    for (int64_t i = 0; i < m; i++) {
        int mx = 0;
        for (int64_t j = 0; j < n; j++) mx = std::max(mx, len[(size_t)(i * n + j)]);
        if (mx > 0) nnz++;
        buf[(size_t)i] = mx > 0 ? mx - 1 : 0;
    }
    if (nnz == 0) {
        PMLG_TRY(identity(K, m));
        for (int64_t i = 0; i < m; i++) pivind[i] = i;
        *nullity_out = m;
        return PMLG_OK;
    }
    int64_t maxdeg = buf[0], diff_shift = shift[0] - buf[0];
    for (int64_t i = 1; i < m; i++) {
        maxdeg = std::max(maxdeg, buf[(size_t)i]);
        diff_shift = std::min(diff_shift, shift[i] - buf[(size_t)i]);
    }
    // order = 1 + max(maxdeg, 1 + (sum(shift) - m * diff_shift - 1) / (m - n)), with
    // C's truncating division as in the reference (:352-356)
    int64_t order = -m * diff_shift - 1;
    for (int64_t i = 0; i < m; i++) order += shift[i];
    order = 1 + order / (m - n);
    order = 1 + std::max(maxdeg, order);

    // the approximant basis, with pmat trimmed to its length
    DevPm pmt;
    PMLG_TRY(window(pm, 0, m, 0, n, plen, pmt));
    int64_t alen = 0;
    PMLG_TRY(alloc(K, m, m, order + 1));
    PMLG_TRY(pmbasis_device(ctx, K.a, K.cap, shift, pmt.a, m, n, plen, order, p_, &alen, st_));

    // rows of the approximant basis that are kernel rows (:361-382)
    std::vector<int> klen;
    PMLG_TRY(lengths(K, klen));
    auto kdeg = [&](int64_t i, int64_t j) { return (int64_t)klen[(size_t)(i * m + j)] - 1; };
    int64_t nullity = 0, sum_pmatdeg = 0;
    bool no_constant_pivot_and_row = true;
    for (int64_t i = 0; i < m; i++) {
        if (shift[i] < order + diff_shift) {
            pivind[nullity++] = i;
        } else {
            if (buf[(size_t)i] == 0 && kdeg(i, i) <= 0) no_constant_pivot_and_row = false;
            sum_pmatdeg += buf[(size_t)i];
            buf[(size_t)(i - nullity)] = i;
        }
    }
    for (int64_t i = nullity; i < m; i++) pivind[i] = buf[(size_t)(i - nullity)];
    // rows and shifts permuted by pivind (nmod_poly_mat_permute_rows)
    PMLG_TRY(permute_rows(K, m, pivind));
    {
        std::vector<int64_t> t(shift, shift + m);
        for (int64_t i = 0; i < m; i++) shift[i] = t[(size_t)pivind[i]];
    }

    // early exit (:392-404)
    if (nullity >= m - n && no_constant_pivot_and_row) {
        int64_t sum_pivdeg = 0;
        for (int64_t i = 0; i < nullity; i++) sum_pivdeg += kdeg(pivind[i], pivind[i]);
        if (sum_pivdeg == sum_pmatdeg) {
            release(pmt);
            *nullity_out = nullity;
            return PMLG_OK;
        }
    }

    // residual of the other rows, its kernel, and the missing kernel rows (:406-441)
    DevPm approx, resid, k2;
    PMLG_TRY(window(K, nullity, m, 0, m, K.cap, approx));
    PMLG_TRY(alloc(resid, m - nullity, n, maxdeg + 1));
    PMLG_TRY(poly_mat_mulmid_device(ctx, resid.a, approx.a, pmt.a, m - nullity, m, n, approx.cap, plen, order,
                                    order + maxdeg + 1, p_, st_));
    release(pmt);
    int64_t nullity2 = 0;
    const int s2 = run(k2, buf.data(), shift + nullity, resid, &nullity2);
    release(resid);
    if (s2 != PMLG_OK || nullity2 == 0) {
        release(k2);
        release(approx);
        *nullity_out = nullity;
        return s2;
    }
    {
        DevPm k2top, prod;
        PMLG_TRY(window(k2, 0, nullity2, 0, m - nullity, k2.cap, k2top));
        PMLG_TRY(mul(k2top, approx, prod));
        PMLG_TRY(set_rows(K, nullity, prod));
        release(k2top);
        release(prod);
    }
    release(k2);
    release(approx);
    for (int64_t i = 0; i < nullity2; i++) pivind[nullity + i] = pivind[nullity + buf[(size_t)i]];

    // merge the two increasing pivot lists, permuting rows, pivots and shifts (:443-468)
    const int64_t tot = nullity + nullity2;
    int64_t i1 = 0, i2 = 0;
    for (int64_t i = 0; i < tot; i++) {
        if (i2 == nullity2 || (i1 < nullity && pivind[i1] < pivind[nullity + i2]))
            buf[(size_t)i] = i1++;
        else
            buf[(size_t)i] = nullity + i2++;
    }
    PMLG_TRY(permute_rows(K, tot, buf.data()));
    std::vector<int64_t> t((size_t)tot);
    for (int64_t i = 0; i < tot; i++) t[(size_t)i] = pivind[i];
    for (int64_t i = 0; i < tot; i++) pivind[i] = t[(size_t)buf[(size_t)i]];
    for (int64_t i = 0; i < tot; i++) t[(size_t)i] = shift[i];
    for (int64_t i = 0; i < tot; i++) shift[i] = t[(size_t)buf[(size_t)i]];
    *nullity_out = tot;
    return PMLG_OK;
}

}  // namespace

}  // namespace pmlg

using namespace pmlg;

extern "C" PMLG_API int pmlg_kernel_zls(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len,
                                        int64_t *pivind, int64_t *shift, const uint64_t *pmat, int64_t m,
                                        int64_t n, int64_t plen, uint64_t p, int64_t *nullity, void *stream)
{
    if (!ctx || m < 0 || n < 0 || plen < 0 || ker_cap < 1 || !nullity || !ker_len) return PMLG_EINVAL;
    if (m > 0 && (!ker || !pivind || !shift)) return PMLG_EINVAL;
    if (m > 0 && n > 0 && plen > 0 && !pmat) return PMLG_EINVAL;
    if (m > LEAF64_MAXDIM) {
        set_error(ctx, "kernel bases support m <= %d (the approximant bases' limit)", LEAF64_MAXDIM);
        return PMLG_EUNSUP;
    }
    if (!h_is_prime(p)) {
        set_error(ctx, "kernel bases need a prime modulus");
        return PMLG_EBADMOD;
    }
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    *nullity = 0;
    *ker_len = 0;
    if (m == 0) return PMLG_OK;
    const size_t kbytes = (size_t)(m * m * ker_cap) * 8;
    if (n == 0 || plen == 0) {
        // the zero matrix (or no columns): the identity, every row a kernel row
        PMLG_CUDA_TRY(cudaMemsetAsync(ker, 0, kbytes, st));
        const uint64_t one = 1;
        for (int64_t i = 0; i < m; i++) {
            PMLG_CUDA_TRY(cudaMemcpyAsync(ker + (i * m + i) * ker_cap, &one, 8, cudaMemcpyHostToDevice, st));
            pivind[i] = i;
        }
        PMLG_CUDA_TRY(cudaStreamSynchronize(st));
        *nullity = m;
        *ker_len = 1;
        return PMLG_OK;
    }
    Kzls z(ctx, p, st);
    DevPm pm;
    pm.a = const_cast<uint64_t *>(pmat);
    pm.r = m; pm.c = n; pm.cap = plen;
    DevPm K;
    int64_t nul = 0;
    int s = z.run(K, pivind, shift, pm, &nul);
    if (s == PMLG_OK) {
        // the kernel rows, trimmed to their length, into the caller's buffer (other rows zero)
        DevPm rows;
        s = z.window(K, 0, nul, 0, m, K.cap, rows);
        int64_t L = 0;
        if (s == PMLG_OK) s = z.max_length(rows, &L);
        if (s == PMLG_OK) {
            *ker_len = L > 0 ? L : 1;
            *nullity = nul;
            if (*ker_len > ker_cap) {
                set_error(ctx, "the kernel basis has length %lld, above the capacity %lld", (long long)*ker_len,
                          (long long)ker_cap);
                s = PMLG_ELEN;
            } else {
                cudaError_t e = cudaMemsetAsync(ker, 0, kbytes, st);
                if (e == cudaSuccess && nul > 0)
                    e = cudaMemcpy2DAsync(ker, (size_t)ker_cap * 8, rows.a, (size_t)rows.cap * 8,
                                          (size_t)std::min(rows.cap, ker_cap) * 8, (size_t)(nul * m),
                                          cudaMemcpyDeviceToDevice, st);
                if (e != cudaSuccess) {
                    set_error(ctx, "kernel basis copy: %s", cudaGetErrorString(e));
                    s = PMLG_ECUDA;
                }
            }
        }
        z.release(rows);
    }
    z.release(K);
    if (s == PMLG_OK) s = device_status(ctx, st);
    if (s == PMLG_OK && cudaStreamSynchronize(st) != cudaSuccess) s = PMLG_ECUDA;
    return s;
}

extern "C" PMLG_API int pmlg_kernel_zls_host(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len,
                                             int64_t *pivind, int64_t *shift, const uint64_t *pmat, int64_t m,
                                             int64_t n, int64_t plen, uint64_t p, int64_t *nullity, void *stream)
{
    if (!ctx || m < 0 || n < 0 || plen < 0 || ker_cap < 1) return PMLG_EINVAL;
    if (m > 0 && !ker) return PMLG_EINVAL;
    if (m > 0 && n > 0 && plen > 0 && !pmat) return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const size_t bP = (size_t)(m * n * plen) * 8, bK = (size_t)(m * m * ker_cap) * 8;
    uint64_t *dP = nullptr, *dK = nullptr;
    PMLG_CUDA_TRY(cudaMallocAsync((void **)&dP, bP + 8, st));
    cudaError_t e = cudaMallocAsync((void **)&dK, bK + 8, st);
    int s = e == cudaSuccess ? PMLG_OK : PMLG_ECUDA;
    if (s == PMLG_OK && bP && cudaMemcpyAsync(dP, pmat, bP, cudaMemcpyHostToDevice, st) != cudaSuccess) s = PMLG_ECUDA;
    if (s == PMLG_OK) s = pmlg_kernel_zls(ctx, dK, ker_cap, ker_len, pivind, shift, dP, m, n, plen, p, nullity, stream);
    if (s == PMLG_OK && bK && cudaMemcpyAsync(ker, dK, bK, cudaMemcpyDeviceToHost, st) != cudaSuccess) s = PMLG_ECUDA;
    if (dK) cudaFreeAsync(dK, st);
    cudaFreeAsync(dP, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && s == PMLG_OK) s = PMLG_ECUDA;
    if (s == PMLG_ECUDA) set_error(ctx, "host-buffer kernel basis: a copy or an allocation failed");
    return s;
}

// ---------------------------------------------------------------------------
// nmod_poly_mat_kernel_via_approx (kernel.c:146-227) and the orientation
// interface nmod_poly_mat_kernel (kernel.c:26-144)
// ---------------------------------------------------------------------------

namespace pmlg {

namespace {

// out entry k <- in entry src[k] (zero when src[k] < 0), out capacity ocap, in capacity icap
__global__ void entry_gather_kernel(uint64_t *__restrict__ out, int64_t ocap, const uint64_t *__restrict__ in,
                                    int64_t icap, const int *__restrict__ src)
{
    const int s = src[blockIdx.x];
    uint64_t *o = out + (int64_t)blockIdx.x * ocap;
    for (int64_t d = threadIdx.x; d < ocap; d += blockDim.x)
        o[d] = (s >= 0 && d < icap) ? in[(int64_t)s * icap + d] : 0ull;
}

int gather_entries(pmlg_ctx *ctx, uint64_t *out, int64_t ocap, const uint64_t *in, int64_t icap,
                   const std::vector<int> &src, cudaStream_t st)
{
    const int64_t ne = (int64_t)src.size();
    if (ne == 0) return PMLG_OK;
    int *d_src = nullptr;
    PMLG_CUDA_TRY(cudaMallocAsync((void **)&d_src, (size_t)ne * sizeof(int), st));
    cudaError_t e = cudaMemcpyAsync(d_src, src.data(), (size_t)ne * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        prof_begin(ctx, "entry_gather", st);
        entry_gather_kernel<<<(unsigned)ne, 128, 0, st>>>(out, ocap, in, icap, d_src);
        prof_end(ctx, st);
        count_launch(ctx);
        e = cudaGetLastError();
    }
    cudaFreeAsync(d_src, st);
    // the index map is a host vector: it must outlive the copy
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error(ctx, "entry gather: %s", cudaGetErrorString(e));
        return PMLG_ECUDA;
    }
    return PMLG_OK;
}

int64_t rank_mod_h(std::vector<uint64_t> a, int64_t r, int64_t c, uint64_t p)
{
    int64_t rank = 0;
    for (int64_t col = 0; col < c && rank < r; col++) {
        int64_t piv = -1;
        for (int64_t i = rank; i < r; i++)
            if (a[(size_t)(i * c + col)] % p) { piv = i; break; }
        if (piv < 0) continue;
        for (int64_t j = 0; j < c; j++) std::swap(a[(size_t)(piv * c + j)], a[(size_t)(rank * c + j)]);
        uint64_t inv = 1, b = a[(size_t)(rank * c + col)] % p, e = p - 2;
        while (e) {
            if (e & 1) inv = (uint64_t)((unsigned __int128)inv * b % p);
            b = (uint64_t)((unsigned __int128)b * b % p);
            e >>= 1;
        }
        for (int64_t i = rank + 1; i < r; i++) {
            const uint64_t f = (uint64_t)((unsigned __int128)(a[(size_t)(i * c + col)] % p) * inv % p);
            if (!f) continue;
            for (int64_t j = col; j < c; j++) {
                const uint64_t t = (uint64_t)((unsigned __int128)f * (a[(size_t)(rank * c + j)] % p) % p);
                const uint64_t x = a[(size_t)(i * c + j)] % p;
                a[(size_t)(i * c + j)] = x >= t ? x - t : x + p - t;
            }
        }
        rank++;
    }
    return rank;
}

int check_kernel_args(pmlg_ctx *ctx, int64_t m, uint64_t p)
{
    if (m > LEAF64_MAXDIM) {
        set_error(ctx, "kernel bases support m <= %d (the approximant bases' limit)", LEAF64_MAXDIM);
        return PMLG_EUNSUP;
    }
    if (!h_is_prime(p)) {
        set_error(ctx, "kernel bases need a prime modulus");
        return PMLG_EBADMOD;
    }
    return PMLG_OK;
}

}  // namespace

}  // namespace pmlg

extern "C" PMLG_API int pmlg_kernel_via_approx(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len,
                                               int64_t *pivind, int64_t *shift, const uint64_t *pmat, int64_t m,
                                               int64_t n, int64_t plen, uint64_t p, int64_t *nullity, void *stream)
{
    if (!ctx || m < 0 || n < 0 || plen < 0 || ker_cap < 1 || !nullity || !ker_len) return PMLG_EINVAL;
    if (m > 0 && (!ker || !pivind || !shift)) return PMLG_EINVAL;
    if (m > 0 && n > 0 && plen > 0 && !pmat) return PMLG_EINVAL;
    PMLG_TRY(check_kernel_args(ctx, m, p));
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    *nullity = 0;
    *ker_len = 1;
    if (m == 0) return PMLG_OK;
    const int64_t ne = m * n, cap0 = plen > 0 ? plen : 1;
    int *d_len = nullptr;
    PMLG_CUDA_TRY(cudaMallocAsync((void **)&d_len, (size_t)(ne > 0 ? ne : 1) * sizeof(int) + 64, st));
    std::vector<int> len;
    int s = (ne > 0 && plen > 0) ? entry_lengths(ctx, pmat, ne, plen, d_len, len, st) : PMLG_OK;
    cudaFreeAsync(d_len, st);
    PMLG_TRY(s);
    int64_t L = 0;
    for (int v : len) L = v > L ? v : L;
    const int64_t d = L - 1;
    const size_t kbytes = (size_t)(m * m * ker_cap) * 8;
    if (d == -1) {   // zero matrix: the identity
        PMLG_CUDA_TRY(cudaMemsetAsync(ker, 0, kbytes, st));
        const uint64_t one = 1;
        for (int64_t i = 0; i < m; i++) {
            PMLG_CUDA_TRY(cudaMemcpyAsync(ker + (i * m + i) * ker_cap, &one, 8, cudaMemcpyHostToDevice, st));
            pivind[i] = i;
        }
        PMLG_CUDA_TRY(cudaStreamSynchronize(st));
        *nullity = m;
        return PMLG_OK;
    }
    if (m == 1) return PMLG_OK;
    if (m <= n) {
        // full row rank of the constant coefficient: empty kernel (:171-184)
        std::vector<uint64_t> c0((size_t)ne);
        PMLG_CUDA_TRY(cudaMemcpy2DAsync(c0.data(), 8, pmat, (size_t)cap0 * 8, 8, (size_t)ne, cudaMemcpyDeviceToHost, st));
        PMLG_CUDA_TRY(cudaStreamSynchronize(st));
        if (rank_mod_h(c0, m, n, p) == m) return PMLG_OK;
    }
    int64_t mn = shift[0], amp = shift[0];
    std::vector<int64_t> rdeg((size_t)m);
    for (int64_t i = 0; i < m; i++) {
        rdeg[(size_t)i] = shift[i];
        if (shift[i] < mn) mn = shift[i];
        else if (shift[i] > amp) amp = shift[i];
    }
    amp -= mn;
    const int64_t order = (m < n ? m : n) * d + amp + d + 1, cap = order + 1;
    uint64_t *K = nullptr;
    PMLG_CUDA_TRY(cudaMallocAsync((void **)&K, (size_t)(m * m * cap) * 8 + 8, st));
    int64_t alen = 0;
    s = pmbasis_device(ctx, K, cap, rdeg.data(), pmat, m, n, cap0, order, p, &alen, st);
    // rows that are kernel rows, moved to the front by swaps (:209-224)
    std::vector<int> src((size_t)(m * m), -1);
    int64_t nul = 0;
    if (s == PMLG_OK) {
        std::vector<int64_t> rowof((size_t)m);
        for (int64_t i = 0; i < m; i++) rowof[(size_t)i] = i;
        for (int64_t i = 0; i < m; i++) {
            if (rdeg[(size_t)i] - shift[i] + amp < order - d) {
                shift[nul] = rdeg[(size_t)i];
                pivind[nul] = i;
                std::swap(rowof[(size_t)nul], rowof[(size_t)i]);
                nul++;
            }
        }
        for (int64_t i = 0; i < nul; i++)
            for (int64_t j = 0; j < m; j++) src[(size_t)(i * m + j)] = (int)(rowof[(size_t)i] * m + j);
        // the length of the kernel rows
        int *d2 = nullptr;
        std::vector<int> klen;
        if (cudaMallocAsync((void **)&d2, (size_t)(m * m) * sizeof(int) + 64, st) != cudaSuccess) s = PMLG_ECUDA;
        if (s == PMLG_OK) s = entry_lengths(ctx, K, m * m, cap, d2, klen, st);
        if (d2) cudaFreeAsync(d2, st);
        int64_t KL = 0;
        if (s == PMLG_OK)
            for (int64_t i = 0; i < nul; i++)
                for (int64_t j = 0; j < m; j++) KL = std::max<int64_t>(KL, klen[(size_t)(rowof[(size_t)i] * m + j)]);
        *ker_len = KL > 0 ? KL : 1;
        *nullity = nul;
        if (s == PMLG_OK && *ker_len > ker_cap) {
            set_error(ctx, "the kernel basis has length %lld, above the capacity %lld", (long long)*ker_len,
                      (long long)ker_cap);
            s = PMLG_ELEN;
        }
        if (s == PMLG_OK) s = gather_entries(ctx, ker, ker_cap, K, cap, src, st);
    }
    cudaFreeAsync(K, st);
    if (s == PMLG_OK) s = device_status(ctx, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && s == PMLG_OK) s = PMLG_ECUDA;
    return s;
}

extern "C" PMLG_API int pmlg_kernel(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len, int64_t *pivind,
                                    int64_t *shift, const uint64_t *pmat, int64_t r, int64_t c, int64_t plen,
                                    uint64_t p, int form, int orient, int64_t *nullity, void *stream)
{
    if (!ctx || r < 0 || c < 0 || plen < 0 || ker_cap < 1 || !nullity || !ker_len) return PMLG_EINVAL;
    if (orient < PMLG_COL_UPPER || orient > PMLG_ROW_LOWER) return PMLG_EINVAL;
    if (form > PMLG_ORD_WEAK_POPOV) {
        set_error(ctx, "kernel bases: forms beyond ordered weak Popov are not implemented (as in kernel.c:34)");
        return PMLG_EUNSUP;
    }
    const bool left = orient == PMLG_ROW_UPPER || orient == PMLG_ROW_LOWER;
    const bool rev = orient == PMLG_ROW_UPPER || orient == PMLG_COL_LOWER;
    const int64_t m = left ? r : c, n = left ? c : r;
    if (m > 0 && (!ker || !pivind)) return PMLG_EINVAL;
    if (r > 0 && c > 0 && plen > 0 && !pmat) return PMLG_EINVAL;
    PMLG_TRY(check_kernel_args(ctx, m, p));
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    *nullity = 0;
    *ker_len = 1;
    if (m == 0) return PMLG_OK;
    const int64_t ne = r * c, cap0 = plen > 0 ? plen : 1;
    // the shift: the caller's, or the row / column degrees (zero for zero rows / columns)
    std::vector<int64_t> sh((size_t)m, 0);
    if (shift) {
        for (int64_t i = 0; i < m; i++) sh[(size_t)i] = shift[i];
    } else if (ne > 0 && plen > 0) {
        int *d_len = nullptr;
        std::vector<int> len;
        PMLG_CUDA_TRY(cudaMallocAsync((void **)&d_len, (size_t)ne * sizeof(int) + 64, st));
        const int s0 = entry_lengths(ctx, pmat, ne, plen, d_len, len, st);
        cudaFreeAsync(d_len, st);
        PMLG_TRY(s0);
        for (int64_t i = 0; i < m; i++)
            for (int64_t j = 0; j < n; j++) {
                const int l = left ? len[(size_t)(i * c + j)] : len[(size_t)(j * c + i)];
                sh[(size_t)i] = std::max<int64_t>(sh[(size_t)i], l > 0 ? l - 1 : 0);
            }
    }
    // the ROW_LOWER problem: transposed for right kernels, rows reversed for ROW_UPPER / COL_LOWER
    std::vector<int> src((size_t)(m * n));
    for (int64_t i = 0; i < m; i++) {
        const int64_t ii = rev ? m - 1 - i : i;
        for (int64_t j = 0; j < n; j++) src[(size_t)(i * n + j)] = (int)(left ? ii * c + j : j * c + ii);
    }
    if (rev) std::reverse(sh.begin(), sh.end());
    uint64_t *M = nullptr, *K = nullptr;
    PMLG_CUDA_TRY(cudaMallocAsync((void **)&M, (size_t)(m * n * cap0) * 8 + 8, st));
    int s = PMLG_OK;
    if (cudaMallocAsync((void **)&K, (size_t)(m * m * ker_cap) * 8 + 8, st) != cudaSuccess) s = PMLG_ECUDA;
    if (s == PMLG_OK && ne > 0) {
        if (plen > 0) s = gather_entries(ctx, M, cap0, pmat, plen, src, st);
        else if (cudaMemsetAsync(M, 0, (size_t)(m * n * cap0) * 8, st) != cudaSuccess) s = PMLG_ECUDA;
    }
    int64_t nul = 0;
    if (s == PMLG_OK)
        s = pmlg_kernel_zls(ctx, K, ker_cap, ker_len, pivind, sh.data(), M, m, n, ne > 0 ? cap0 : 0, p, &nul, stream);
    if (s == PMLG_OK) {
        if (rev && nul > 0) {
            // kernel rows reversed (and their shifts), columns reversed, pivots mirrored (:91-103)
            std::reverse(sh.begin(), sh.begin() + nul);
            for (int64_t i = 0; i < nul / 2; i++) {
                const int64_t t = m - 1 - pivind[i];
                pivind[i] = m - 1 - pivind[nul - 1 - i];
                pivind[nul - 1 - i] = t;
            }
            if (nul % 2) pivind[nul / 2] = m - 1 - pivind[nul / 2];
        }
        // final entry (a, b): rows a < nullity of the (reversed) kernel, transposed for right kernels
        std::vector<int> fsrc((size_t)(m * m), -1);
        for (int64_t a = 0; a < m; a++)
            for (int64_t b = 0; b < m; b++) {
                const int64_t i = left ? a : b, j = left ? b : a;   // kernel row i, column j
                if (i >= nul) continue;
                fsrc[(size_t)(a * m + b)] = (int)(rev ? (nul - 1 - i) * m + (m - 1 - j) : i * m + j);
            }
        s = gather_entries(ctx, ker, ker_cap, K, ker_cap, fsrc, st);
        *nullity = nul;
        if (shift)
            for (int64_t i = 0; i < m; i++) shift[i] = sh[(size_t)i];
    }
    cudaFreeAsync(M, st);
    if (K) cudaFreeAsync(K, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && s == PMLG_OK) s = PMLG_ECUDA;
    return s;
}
