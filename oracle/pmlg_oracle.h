/*
 * pmlg_oracle.h -- CPU restatement of PML's evaluation/interpolation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path is
 * compared against, and the CPU baseline that bench.py times beside it.  The
 * product library (libpmlg) never links, loads or calls it.
 *
 * Parity status:
 *   - products, middle products, matrix products, dot products and CRT have a
 *     unique answer mod p; the schoolbook routines here are pinned against an
 *     independent Python big-integer restatement (tests/golden/make_golden.py)
 *     and against the reference tests' known answers (all-(p-1) worst case of
 *     flint-extras/src/nmod32_vec/test/t-dot.c, x^k identities).
 *   - mbasis/pmbasis follow flint-extras/src/nmod_mat_poly_extra/
 *     nmod_mat_poly_mbasis.c:116-378 and nmod_poly_mat_extra/approximant_basis.c:33-69
 *     step for step; the reference's own tests pin them only by the property
 *     check restated in orc_is_approximant_basis (nmod_poly_mat_extra/
 *     verification.c:21-116), which is what the tests here apply.  Bit values of
 *     pmbasis are therefore "parity unpinned" against FLINT itself (FLINT is not
 *     available to build here).
 *
 * Layouts (all dense, zero padded):
 *   matrix       : row-major, M[i*c + j]
 *   poly matrix  : entry-major, P[(i*c + j)*len + d]   (coefficient d of entry (i,j))
 * Coefficients are uint64_t in [0, p), p any modulus 2 <= p < 2^64.
 */
#ifndef PMLG_ORACLE_H
#define PMLG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- seeded generator: SplitMix64, uniform [0,p) by rejection ---- */
uint64_t orc_splitmix64(uint64_t *state);
void orc_rand_vec(uint64_t *v, int64_t n, uint64_t p, uint64_t seed);
void orc_rand_vec_u32(uint32_t *v, int64_t n, uint64_t p, uint64_t seed);

/* ---- scalars ---- */
uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t p);
uint64_t orc_powmod(uint64_t a, uint64_t e, uint64_t p);
uint64_t orc_invmod(uint64_t a, uint64_t p);
int orc_is_prime(uint64_t n);
/* seeded random prime of exactly `bits` bits (2 <= bits <= 63) */
uint64_t orc_rand_prime(int bits, uint64_t seed);
/* nmod_find_root: smallest q >= 2 of multiplicative order >= n (0 if none);
 * flint-extras/src/nmod_extra/nmod_find_root.c:21-38 */
uint64_t orc_find_root(uint64_t n, uint64_t p);

/* ---- matrices ---- */
/* C (r x c) = A (r x k) * B (k x c) mod p; FLINT nmod_mat_mul semantics */
void orc_nmod_mat_mul(uint64_t *C, const uint64_t *A, const uint64_t *B,
                      int64_t r, int64_t k, int64_t c, uint64_t p);
/* batch of nbatch independent products, uint32 storage (p < 2^32) */
void orc_nmod_mat_mul_batch_u32(uint32_t *C, const uint32_t *A, const uint32_t *B,
                                int64_t nbatch, int64_t r, int64_t k, int64_t c,
                                uint64_t p, int nthreads);
/* rank of a dense matrix mod p (prime) */
int64_t orc_nmod_mat_rank(const uint64_t *A, int64_t r, int64_t c, uint64_t p);
/* reduced row echelon form in place; returns rank (prime p) */
int64_t orc_nmod_mat_rref(uint64_t *A, int64_t r, int64_t c, uint64_t p);
/* nmod_mat_left_nullspace_compact, left_nullspace.c:42-102:
 * A is m x n; X receives nullity x rank (row-major, rank columns);
 * perm[0..rank) = row rank profile (increasing), perm[rank..m) = complement.
 * Returns nullity. */
int64_t orc_left_nullspace_compact(uint64_t *X, int64_t *perm,
                                   const uint64_t *A, int64_t m, int64_t n, uint64_t p);

/* ---- polynomial matrices ---- */
/* max length over entries (trailing zero coefficients ignored) */
int64_t orc_pm_max_length(const uint64_t *P, int64_t r, int64_t c, int64_t cap);
/* C = A * B; A r x k of capacity len1, B k x c of capacity len2; C capacity
 * len1+len2-1 (fully written). Schoolbook. */
void orc_poly_mat_mul(uint64_t *C, const uint64_t *A, const uint64_t *B,
                      int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                      uint64_t p, int nthreads);
/* nmod_poly_mat_mulmid semantics (mulmid.c:499-541): res = (A*B mod x^nhi) div x^nlo.
 * res has capacity (nhi - nlo) per entry and is fully written (zeros beyond the
 * clamped length).  Returns the clamped output length max(0, min(nhi, L1+L2-1) - nlo),
 * where L1, L2 are the max lengths of A and B.  Schoolbook. */
int64_t orc_poly_mat_mulmid(uint64_t *res, const uint64_t *A, const uint64_t *B,
                            int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                            int64_t nlo, int64_t nhi, uint64_t p, int nthreads);

/* Evaluation/interpolation product on the CPU (the algorithm of
 * nmod_poly_mat_extra/mul_geometric.c:32-119 with evaluation at roots of unity
 * instead of a geometric progression): forward NTT of every entry, one matrix
 * product per point, inverse NTT.  p must be an NTT prime < 2^30 with
 * 2^ceil(log2(len1+len2-1)) | p-1.  This is the CPU baseline "port". */
int orc_poly_mat_mul_ntt(uint64_t *C, const uint64_t *A, const uint64_t *B,
                         int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                         uint64_t p, int nthreads);
/* C = A * B mod any p >= 2 by NTT products modulo up to 6 primes below 2^30 and
 * Garner's CRT (the multi-prime design of nmod_poly_mat_mul_3_primes.bak:59-153);
 * -1 when the product needs more primes or a transform beyond 2^20. */
int orc_poly_mat_mul_crt(uint64_t *C, const uint64_t *A, const uint64_t *B,
                         int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                         uint64_t p, int nthreads);

/* ---- approximant bases ---- */
/* nmod_poly_mat_mbasis (approximant_basis.c:18-31 -> nmod_mat_poly_mbasis.c:116-378).
 * F: m x n, capacity flen; appbas: m x m of capacity order+1 (fully written);
 * shift: m entries, in = input shift, out = shifted row degree.
 * Returns the max length of appbas. */
int64_t orc_mbasis(uint64_t *appbas, int64_t *shift, const uint64_t *F,
                   int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p);
/* nmod_poly_mat_pmbasis (approximant_basis.c:33-69) with leaf threshold `thres`
 * (PMBASIS_THRES = 32 in the reference). Same conventions as orc_mbasis. */
int64_t orc_pmbasis(uint64_t *appbas, int64_t *shift, const uint64_t *F,
                    int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p,
                    int64_t thres, int nthreads);
/* nmod_poly_mat_is_approximant_basis (verification.c:21-116), ROW_LOWER.
 * Returns a bitmask of failed checks (0 = success):
 *   1 not ordered weak Popov, 2 residual not zero mod x^order,
 *   4 det degree != sum of diagonal degrees, 8 [P(0) | C] not of full rank.
 * Check 4 is evaluated at sum(rowdeg)+1 points and is skipped (not failed)
 * when p is too small to provide them. */
int orc_is_approximant_basis(const uint64_t *appbas, int64_t alen,
                             const uint64_t *F, int64_t flen,
                             int64_t m, int64_t n, int64_t order,
                             const int64_t *shift_in, uint64_t p);

/* ---- dot products (flint-extras/src/nmod_vec_extra, nmod32_vec) ---- */
/* sum v1[i]*v2[i] mod p for arbitrary 64-bit entries (not assumed reduced),
 * nmod_vec_dot_product_unbalanced, nmod_vec_dot_product.c:136-147 */
uint64_t orc_nmod_vec_dot(const uint64_t *v1, const uint64_t *v2, int64_t len, uint64_t p);
void orc_nmod_vec_dot_multi(uint64_t *uv, const uint64_t *u, const uint64_t *v, int64_t len, int64_t k,
                            uint64_t p, int nthreads);
/* 32-bit storage, _nmod32_vec_dot_split, nmod32_vec/dot_split.c:18-47 */
uint32_t orc_nmod32_vec_dot(const uint32_t *v1, const uint32_t *v2, int64_t len, uint64_t p);
/* exact integer dot product in 3 limbs, nmod_vec_integer_dot_product.c:13 */
void orc_integer_dot(uint64_t res[3], const uint64_t *v1, const uint64_t *v2, int64_t len);
/* mv[i] = sum_j mat[i*stride + j] * vec[j] mod p, _nmod32_vec_mdot_split (mdot_split.c:17) */
void orc_nmod32_vec_mdot(uint32_t *mv, const uint32_t *mat, const uint32_t *vec,
                         int64_t nrows, int64_t len, int64_t stride, uint64_t p);

/* ---- multimodular reduction / CRT (nmod_extra/nmod_multimod_CRT_*.c) ---- */
/* residues[j*nb + i] = input[i] mod primes[j] */
void orc_multimod_reduce(uint64_t *residues, const uint64_t *input, int64_t nb,
                         const uint64_t *primes, int nprimes);
/* out[i] = CRT(residues[j*nb + i], j < nprimes) mod p (the CRT value is taken in
 * [0, prod primes)) */
void orc_multimod_crt(uint64_t *out, const uint64_t *residues, int64_t nb,
                      const uint64_t *primes, int nprimes, uint64_t p);

/* ---- kernel basis (flint-extras/src/nmod_poly_mat_extra/kernel.c) ---- */
/* nmod_poly_mat_kernel_zls_approx (kernel.c:232-480), left kernel (ROW_LOWER) of
 * the m x n matrix pmat (entry capacity plen).  shift: m entries, in = s, out: the
 * s-row degrees of the kernel rows in [0, nullity); pivind: m entries, out: the
 * s-pivot indices of the kernel rows in [0, nullity).  *ker receives an m x m
 * matrix (free it with orc_free) of capacity *klen whose rows [0, nullity) are the
 * kernel basis, in s-ordered weak Popov form with increasing pivots; its other
 * rows are zero.  Returns the nullity. */
int64_t orc_kernel_zls(uint64_t **ker, int64_t *klen, int64_t *pivind, int64_t *shift,
                       const uint64_t *pmat, int64_t m, int64_t n, int64_t plen, uint64_t p,
                       int nthreads);
/* nmod_poly_mat_kernel_via_approx (kernel.c:146-227): same conventions as
 * orc_kernel_zls. */
int64_t orc_kernel_via_approx(uint64_t **ker, int64_t *klen, int64_t *pivind, int64_t *shift,
                              const uint64_t *pmat, int64_t m, int64_t n, int64_t plen, uint64_t p,
                              int nthreads);
/* nmod_poly_mat_kernel (kernel.c:26-144), form ORD_WEAK_POPOV, orientation orient
 * (COL_UPPER 0, COL_LOWER 1, ROW_UPPER 2, ROW_LOWER 3).  pmat: r x c, capacity plen.
 * Left kernels: *ker is r x r, the basis in its first nullity rows; right kernels:
 * c x c, the basis in its first nullity columns; other rows / columns zero.  shift
 * NULL: the default (row or column degrees, zero for zero rows or columns). */
int64_t orc_kernel(uint64_t **ker, int64_t *klen, int64_t *pivind, int64_t *shift, const uint64_t *pmat,
                   int64_t r, int64_t c, int64_t plen, uint64_t p, int orient, int nthreads);
void orc_free(void *ptr);

/* ---- shifted Popov approximant basis ---- */
/* popov_pmbasis (ntl-extras/mat_lzz_pX_extra/src/mat_lzz_pX_pmbasis.cpp:1527-1557):
 * pmbasis with shift s, then with shift s - rdeg_s, then the product by the inverse of
 * the second basis' row leading matrix.  appbas: m x m, capacity order + 1; shift: in s,
 * out the s-row degree.  Returns appbas' length. */
int64_t orc_popov_pmbasis(uint64_t *appbas, int64_t *shift, const uint64_t *F, int64_t m, int64_t n,
                          int64_t flen, int64_t order, uint64_t p, int nthreads);

/* ---- truncated inverse and Dixon lifting (nmod_poly_mat_extra/nmod_poly_mat_dixon.c) ---- */
/* S (n x n, capacity order + 1) = A^-1 mod x^order (:32-80); returns 1, or 0 when A(0) is
 * singular (S untouched). */
int orc_inv_trunc(uint64_t *S, const uint64_t *A, int64_t n, int64_t alen, int64_t order, uint64_t p,
                  int nthreads);
/* X (n x m, capacity ceil(sigma / order) * order) with A X = B mod x^sigma (:92-143);
 * returns 1, or 0 when A(0) is singular. */
int orc_dixon(uint64_t *X, const uint64_t *A, const uint64_t *B, int64_t n, int64_t m, int64_t alen,
              int64_t blen, int64_t order, int64_t sigma, uint64_t p, int nthreads);

/* ---- layout conversions ---- */
/* nmod_mat_poly_set_trunc_from_poly_mat (nmod_mat_poly_set_from.c:31-52):
 * out[k][i][j] = in[(i*c + j)*ld + k] for k < min(order, len), zero up to out_cap;
 * returns the normalised length (last nonzero coefficient matrix + 1). */
int64_t orc_poly_mat_to_mat_poly(uint64_t *out, int64_t out_cap, const uint64_t *in, int64_t r, int64_t c,
                                 int64_t ld, int64_t len, int64_t order);
/* nmod_poly_mat_set_trunc_from_mat_poly (nmod_poly_mat_utils.c:185-210):
 * out[(i*c + j)*out_cap + k] = in[k][i][j] for k < min(order, len), zero up to out_cap. */
void orc_mat_poly_to_poly_mat(uint64_t *out, int64_t out_cap, const uint64_t *in, int64_t r, int64_t c,
                              int64_t len, int64_t order);

#ifdef __cplusplus
}
#endif

#endif
