// polymat.cuh -- evaluation / pointwise / interpolation pipeline shared by the
// product, the middle product, the batched products and pmbasis.
#pragma once
#include "pmlg_internal.cuh"

#include <vector>

namespace pmlg {

// One product job in device memory.  Coefficients [lo, lo + cnt) of the
// length-N cyclic convolution of A (entries A + e*lda + a_off, a_len
// coefficients) and B (likewise) are written to C (entry stride ldc, capacity
// c_cap, zero beyond cnt).  N = 2^lg must satisfy N >= lo + cnt and
// N >= a_len + b_len - 1 - lo so that no wrapped term lands in the window.
struct ProductJob
{
    int64_t r, k, c;
    const uint64_t *A;
    int64_t lda, a_off, a_len;
    const uint64_t *B;
    int64_t ldb, b_off, b_len;
    uint64_t *C;
    int64_t ldc, c_cap;
    int64_t lo, cnt;
    int lg;
    uint64_t p;
};

// Bytes of scratch one job needs.
size_t product_scratch_bytes(const ProductJob &j, const CrtPlan &plan);

// Evaluations of a left operand kept across products with the same left operand
// (the precomputation of _nmod_poly_mat_mul_geometric_precomp, mul_geometric.c:32-119):
// `words` words of device memory that hold, once `valid`, the forward transforms at
// size 2^lg, for the NTT primes q[0..t), of the r x k operand read at (a, lda, a_off, a_len).
// A product that differs in any of these transforms its operand again into the
// buffer.  The caller keeps the operand's contents unchanged while the cache is valid.
struct EvalCache
{
    uint32_t *ea = nullptr;
    size_t words = 0;
    bool valid = false;
    int lg = 0, t = 0;
    uint32_t q[kMaxPrimes] = {};
    const uint64_t *a = nullptr;
    int64_t r = 0, k = 0, lda = 0, a_off = 0, a_len = 0;
};

// Runs one job on the stream using `scratch` (at least product_scratch_bytes); with a
// cache, the left operand's evaluations come from (or are stored into) it.
int product_run(pmlg_ctx *ctx, const ProductJob &j, const CrtPlan &plan, void *scratch,
                int form, cudaStream_t st, EvalCache *ca = nullptr);

// Transform size for a middle product window after the input trimming of
// mulmid.c:516-556: returns lg, and adjusts offsets/lengths/window in place.
int mulmid_prepare(ProductJob &j, int64_t len1, int64_t len2, int64_t nlo, int64_t nhi);

int lg_for(int64_t n);

// Dense device products (entry strides len1, len2; C: len1 + len2 - 1, res: nhi - nlo).
int poly_mat_mul_device(pmlg_ctx *ctx, uint64_t *C, const uint64_t *A, const uint64_t *B, int64_t r,
                        int64_t k, int64_t c, int64_t len1, int64_t len2, uint64_t p, cudaStream_t st,
                        EvalCache *ca = nullptr);
int poly_mat_mulmid_device(pmlg_ctx *ctx, uint64_t *res, const uint64_t *A, const uint64_t *B,
                           int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2, int64_t nlo,
                           int64_t nhi, uint64_t p, cudaStream_t st, EvalCache *ca = nullptr);

// pmbasis on device buffers (appbas capacity cap >= order + 1, F entry stride flen),
// shift on the host; *len is appbas' exact max length.
int pmbasis_device(pmlg_ctx *ctx, uint64_t *appbas, int64_t cap, int64_t *shift, const uint64_t *F,
                   int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p, int64_t *len,
                   cudaStream_t st);

// Length (last nonzero coefficient + 1) of each of nent entries of capacity cap, into
// len on the host (d_out: nent ints of device scratch; synchronises the stream).
int entry_lengths(pmlg_ctx *ctx, const uint64_t *P, int64_t nent, int64_t cap, int *d_out, std::vector<int> &len,
                  cudaStream_t st);

}  // namespace pmlg
