// popov.cu -- shifted Popov approximant bases: popov_pmbasis
// (ntl-extras/mat_lzz_pX_extra/src/mat_lzz_pX_pmbasis.cpp:1527-1557; listed as a TODO
// in flint-extras/src/nmod_poly_mat_approximant.h:337-348).
//
// pmbasis with shift s gives the s-row degree rdeg; pmbasis again with shift s - rdeg
// (minus the pivot degrees) gives a basis that is s-Popov up to a constant
// transformation; multiplying on the left by the inverse of its (s - rdeg)-row leading
// matrix yields the s-Popov approximant basis, which is unique.  Both pmbasis calls
// and the final product run on the device; the host reads entry lengths, gathers the
// m x m leading matrix and inverts it (m <= 64).
#include "pmlg_internal.cuh"
#include "polymat.cuh"

#include <vector>

namespace pmlg {

namespace {

// lm[e] = P[e * cap + k[e]] (0 when k[e] < 0)
__global__ void gather_coeffs_kernel(const uint64_t *__restrict__ P, int64_t cap, const int64_t *__restrict__ k,
                                     int64_t nent, uint64_t *__restrict__ lm)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nent) lm[e] = (k[e] >= 0 && k[e] < cap) ? P[e * cap + k[e]] : 0ull;
}

uint64_t mulmod_h(uint64_t a, uint64_t b, uint64_t p)
{
    return (uint64_t)((unsigned __int128)a * b % p);
}

uint64_t powmod_h(uint64_t a, uint64_t e, uint64_t p)
{
    uint64_t r = 1 % p;
    while (e) {
        if (e & 1) r = mulmod_h(r, a, p);
        a = mulmod_h(a, a, p);
        e >>= 1;
    }
    return r;
}

// inverse of the m x m matrix M mod p by Gauss-Jordan; false when singular
bool invert_h(std::vector<uint64_t> &M, int64_t m, uint64_t p, std::vector<uint64_t> &inv)
{
    std::vector<uint64_t> a((size_t)(m * 2 * m), 0);
    for (int64_t i = 0; i < m; i++) {
        for (int64_t j = 0; j < m; j++) a[(size_t)(i * 2 * m + j)] = M[(size_t)(i * m + j)];
        a[(size_t)(i * 2 * m + m + i)] = 1;
    }
    for (int64_t c = 0; c < m; c++) {
        int64_t piv = -1;
        for (int64_t i = c; i < m; i++)
            if (a[(size_t)(i * 2 * m + c)]) { piv = i; break; }
        if (piv < 0) return false;
        if (piv != c)
            for (int64_t j = 0; j < 2 * m; j++) std::swap(a[(size_t)(piv * 2 * m + j)], a[(size_t)(c * 2 * m + j)]);
        const uint64_t iv = powmod_h(a[(size_t)(c * 2 * m + c)], p - 2, p);
        for (int64_t j = 0; j < 2 * m; j++) a[(size_t)(c * 2 * m + j)] = mulmod_h(a[(size_t)(c * 2 * m + j)], iv, p);
        for (int64_t i = 0; i < m; i++) {
            if (i == c) continue;
            const uint64_t f = a[(size_t)(i * 2 * m + c)];
            if (!f) continue;
            for (int64_t j = 0; j < 2 * m; j++) {
                const uint64_t t = mulmod_h(f, a[(size_t)(c * 2 * m + j)], p);
                uint64_t &x = a[(size_t)(i * 2 * m + j)];
                x = x >= t ? x - t : x + p - t;
            }
        }
    }
    inv.assign((size_t)(m * m), 0);
    for (int64_t i = 0; i < m; i++)
        for (int64_t j = 0; j < m; j++) inv[(size_t)(i * m + j)] = a[(size_t)(i * 2 * m + m + j)];
    return true;
}

}  // namespace

}  // namespace pmlg

using namespace pmlg;

extern "C" PMLG_API int pmlg_popov_pmbasis(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                                           const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                                           uint64_t p, int64_t *appbas_len, void *stream)
{
    if (!ctx || !shift || m <= 0 || n <= 0 || flen < 0 || order < 0 || appbas_cap < order + 1 || !appbas)
        return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    // first call: the s-row degree
    std::vector<int64_t> rdeg(shift, shift + m), pshift((size_t)m), t((size_t)m);
    int64_t len = 0;
    PMLG_TRY(pmbasis_device(ctx, appbas, appbas_cap, rdeg.data(), F, m, n, flen, order, p, &len, st));
    // second call with shift s - rdeg_s
    for (int64_t i = 0; i < m; i++) {
        pshift[(size_t)i] = shift[i] - rdeg[(size_t)i];
        t[(size_t)i] = pshift[(size_t)i];
        shift[i] = rdeg[(size_t)i];
    }
    PMLG_TRY(pmbasis_device(ctx, appbas, appbas_cap, pshift.data(), F, m, n, flen, order, p, &len, st));

    // the t-row leading matrix: row i holds the coefficients of degree rdeg_t(i) - t[j]
    const int64_t ne = m * m;
    void *scratch = nullptr;
    const size_t sb = (size_t)ne * (sizeof(int) + 2 * sizeof(int64_t) + 8) + 256;
    PMLG_CUDA_TRY(cudaMallocAsync(&scratch, sb, st));
    int *d_len = (int *)scratch;
    int64_t *d_k = (int64_t *)((char *)scratch + ((ne * sizeof(int) + 15) & ~(size_t)15));
    uint64_t *d_lm = (uint64_t *)(d_k + ne);
    uint64_t *d_inv = d_lm + ne;
    std::vector<int> elen;
    int s = entry_lengths(ctx, appbas, ne, appbas_cap, d_len, elen, st);
    std::vector<int64_t> k((size_t)ne, -1);
    if (s == PMLG_OK) {
        for (int64_t i = 0; i < m; i++) {
            bool any = false;
            int64_t rd = 0;
            for (int64_t j = 0; j < m; j++) {
                const int d = elen[(size_t)(i * m + j)] - 1;
                if (d >= 0 && (!any || d + t[(size_t)j] > rd)) { rd = d + t[(size_t)j]; any = true; }
            }
            for (int64_t j = 0; j < m; j++) k[(size_t)(i * m + j)] = any ? rd - t[(size_t)j] : -1;
        }
        if (cudaMemcpyAsync(d_k, k.data(), (size_t)ne * sizeof(int64_t), cudaMemcpyHostToDevice, st) != cudaSuccess)
            s = PMLG_ECUDA;
    }
    std::vector<uint64_t> lm((size_t)ne), inv;
    if (s == PMLG_OK) {
        gather_coeffs_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(appbas, appbas_cap, d_k, ne, d_lm);
        count_launch(ctx);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(lm.data(), d_lm, (size_t)ne * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            s = PMLG_ECUDA;
    }
    if (s == PMLG_OK && !invert_h(lm, m, p, inv)) {
        set_error(ctx, "popov_pmbasis: the row leading matrix is singular");
        s = PMLG_EUNSUP;
    }
    if (s == PMLG_OK) {
        // appbas <- inv * appbas, over the basis' length
        int64_t L = 0;
        for (int v : elen) L = v > L ? v : L;
        if (L < 1) L = 1;
        uint64_t *prod = nullptr;
        if (cudaMemcpyAsync(d_inv, inv.data(), (size_t)ne * 8, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMallocAsync((void **)&prod, (size_t)(ne * L) * 8 + 8, st) != cudaSuccess) {
            s = PMLG_ECUDA;
        } else {
            // the product reads appbas with entry stride L: compact it into prod first, then
            // multiply into a second buffer
            uint64_t *compact = nullptr;
            if (cudaMallocAsync((void **)&compact, (size_t)(ne * L) * 8 + 8, st) != cudaSuccess ||
                cudaMemcpy2DAsync(compact, (size_t)L * 8, appbas, (size_t)appbas_cap * 8, (size_t)L * 8, (size_t)ne,
                                  cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                s = PMLG_ECUDA;
            if (s == PMLG_OK) s = poly_mat_mul_device(ctx, prod, d_inv, compact, m, m, m, 1, L, p, st);
            if (s == PMLG_OK &&
                (cudaMemsetAsync(appbas, 0, (size_t)(ne * appbas_cap) * 8, st) != cudaSuccess ||
                 cudaMemcpy2DAsync(appbas, (size_t)appbas_cap * 8, prod, (size_t)L * 8, (size_t)L * 8, (size_t)ne,
                                   cudaMemcpyDeviceToDevice, st) != cudaSuccess))
                s = PMLG_ECUDA;
            if (compact) cudaFreeAsync(compact, st);
            cudaFreeAsync(prod, st);
        }
        if (s == PMLG_OK && appbas_len) {
            std::vector<int> flen2;
            s = entry_lengths(ctx, appbas, ne, appbas_cap, d_len, flen2, st);
            int64_t L2 = 0;
            for (int v : flen2) L2 = v > L2 ? v : L2;
            *appbas_len = L2;
        }
    }
    cudaFreeAsync(scratch, st);
    if (s == PMLG_ECUDA) set_error(ctx, "popov_pmbasis: a device copy or allocation failed");
    if (s == PMLG_OK) s = device_status(ctx, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && s == PMLG_OK) s = PMLG_ECUDA;
    return s;
}
