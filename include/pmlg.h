/*
 * pmlg.h -- C ABI of pml-gb300: the evaluation/interpolation hot path of PML
 * (polynomial matrices over Z/pZ) on one GB300 (sm_103a).
 *
 * Every entry point is a plain C function over plain pointers and sizes.
 * Functions named *_host take host buffers and do the host<->device copies
 * themselves; all others take DEVICE pointers and run stream-ordered on the
 * given cudaStream_t (passed as void*, NULL = legacy default stream).
 *
 * Layouts (dense, zero padded, the coefficient arrays of FLINT's nmod_poly
 * entries laid side by side):
 *   matrix       : row-major, M[i*c + j]
 *   poly matrix  : entry-major, P[(i*c + j)*len + d] = coefficient d of entry (i,j)
 * Coefficients are uint64_t in [0, p) (FLINT ulong), 2 <= p < 2^64, unless a
 * function says uint32_t.  Inputs must be reduced mod p, as FLINT requires.
 *
 * Return value: PMLG_OK (0) or a PMLG_E* status; nothing aborts.  After an
 * error, pmlg_ctx_last_error() describes it.
 */
#ifndef PMLG_H
#define PMLG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PMLG_API __attribute__((visibility("default")))
#else
#define PMLG_API
#endif

typedef struct pmlg_ctx pmlg_ctx;

enum pmlg_status_code
{
    PMLG_OK = 0,
    PMLG_EINVAL = 1,     /* bad argument (negative size, null pointer, ...) */
    PMLG_EBADMOD = 2,    /* modulus not supported by this entry point */
    PMLG_ENOROOT = 3,    /* no root of unity of the needed order */
    PMLG_ELEN = 4,       /* length beyond the supported transform size */
    PMLG_EALIAS = 5,     /* output overlaps an input where that is not allowed */
    PMLG_ETIMEOUT = 6,   /* a bounded device wait gave up */
    PMLG_ECUDA = 7,      /* CUDA runtime error */
    PMLG_ENOMEM = 8,     /* device or host allocation failed */
    PMLG_EUNSUP = 9      /* shape outside what this build supports */
};

/* Which kernel form computes the pointwise matrix products. */
enum pmlg_form
{
    PMLG_FORM_AUTO = 0,       /* per shape class, the form measured fastest (pmlg_ctx_set_tuning) */
    PMLG_FORM_CUDA_CORE = 1,  /* uint64 multiply-accumulate with delayed reduction */
    PMLG_FORM_INT8_TC = 2,    /* 8-bit limbs on the INT8 tensor cores (mma.sync, s32 accumulate) */
    PMLG_FORM_F16_TC = 3      /* exact small signed digits in FP16 on tcgen05 (FP32 accumulate, all
                                 partial sums below 2^22 so every step is exact) */
};

/* Orientations and forms of polynomial matrices, with the values of the reference's
 * orientation_t and poly_mat_form_t (flint-extras/src/nmod_poly_mat_forms.h:57-104). */
enum pmlg_orientation
{
    PMLG_COL_UPPER = 0,
    PMLG_COL_LOWER = 1,
    PMLG_ROW_UPPER = 2,
    PMLG_ROW_LOWER = 3
};
enum pmlg_poly_mat_form
{
    PMLG_NONE = 0,
    PMLG_REDUCED = 1,
    PMLG_WEAK_POPOV = 2,
    PMLG_ORD_WEAK_POPOV = 3,
    PMLG_POPOV = 4
};

/* ---------------------------------------------------------------------- */
/* context                                                                 */
/* ---------------------------------------------------------------------- */

/* Creates a context on `device`: holds the NTT tables per (prime, length), the
 * device scratch and pinned staging buffers.  One context per host thread. */
PMLG_API int pmlg_ctx_create(pmlg_ctx **ctx, int device);
PMLG_API int pmlg_ctx_destroy(pmlg_ctx *ctx);
PMLG_API int pmlg_ctx_set_form(pmlg_ctx *ctx, int form);
/* PMLG_FORM_AUTO measures the three forms on the first product of each shape class
 * (r, k, c, number of points rounded up to a power of two) and keeps the fastest for
 * the class; on = 0 makes AUTO take the FP16 form without measuring. */
PMLG_API int pmlg_ctx_set_tuning(pmlg_ctx *ctx, int on);
/* the form AUTO chose for a shape class, PMLG_FORM_AUTO when none was measured yet,
 * -PMLG_EINVAL for a shape outside 1..64 */
PMLG_API int pmlg_ctx_tuned_form(const pmlg_ctx *ctx, int r, int k, int c, int64_t npts);
/* pmlg_poly_mat_mul_batch: on (the default), a batch called again with the same jobs is
 * captured into a CUDA graph on its second call and replayed on later ones; a capture that
 * fails falls back to direct launches and leaves replay off until this is called again */
PMLG_API int pmlg_ctx_set_batch_graphs(pmlg_ctx *ctx, int on);
/* pmbasis leaf order (mbasis below it); 0 restores the tuned default */
PMLG_API int pmlg_ctx_set_leaf_order(pmlg_ctx *ctx, int64_t order);
/* number of kernels this context has launched so far */
PMLG_API unsigned long long pmlg_ctx_launch_count(const pmlg_ctx *ctx);
PMLG_API const char *pmlg_ctx_last_error(const pmlg_ctx *ctx);
/* Failure detection: every device-side wait of the kernels (mbarrier phases,
 * published eliminations) is bounded; a wait that gives up sets the context's
 * device error word and the kernel returns.  device_status synchronises
 * `stream`, reads and clears the word, and returns PMLG_ETIMEOUT if it was set
 * (the results since the previous check are then invalid).  The host-buffer
 * entry points and pmbasis/mbasis check it before they return; callers of the
 * stream-ordered device entry points call it when they synchronise.  No
 * reference counterpart: the reference has no device and aborts on errors. */
PMLG_API int pmlg_ctx_device_status(pmlg_ctx *ctx, void *stream);
/* Diagnostic: a kernel waits (at most wait_ns, <= 1 s) on an mbarrier phase
 * that nothing completes and reports through the error word; returns
 * PMLG_ETIMEOUT from device_status, with the context still usable. */
PMLG_API int pmlg_ctx_selftest_timeout(pmlg_ctx *ctx, unsigned long long wait_ns, void *stream);
/* Kernel timing (tracing): when on, every kernel launched through the context
 * is bracketed by CUDA events recorded on its own stream.  set_profiling also
 * clears the records.  profile_read synchronises on the recorded events and
 * returns, per kernel name, the summed device time in ms and the launch count
 * (names '\n'-separated in `names`).  Plays the role of the reference's
 * MBASIS_PROFILE timers (nmod_mat_poly_mbasis.c:9-57). */
PMLG_API int pmlg_ctx_set_profiling(pmlg_ctx *ctx, int on);
PMLG_API int pmlg_ctx_profile_read(pmlg_ctx *ctx, char *names, size_t names_len, double *ms,
                                   unsigned long long *counts, int max_kernels, int *n_out);
PMLG_API const char *pmlg_strerror(int status);

/* ---------------------------------------------------------------------- */
/* L2: batched matrix products mod p at the evaluation points              */
/* ---------------------------------------------------------------------- */

/* C[b] = A[b] * B[b] mod p for b < nbatch; A[b] r x k, B[b] k x c, C[b] r x c,
 * row-major, stored contiguously batch after batch, uint32 storage.
 * Requires p < 2^30 (any p, prime or not).  Replaces the per-point FLINT
 * nmod_mat_mul loop of flint-extras/src/nmod_poly_mat_extra/mul_geometric.c:95-96
 * (and mulmid.c:105-106, 200-201).  Uses the context's form. */
PMLG_API int pmlg_nmod_mat_mul_batch_u32(pmlg_ctx *ctx, uint32_t *C, const uint32_t *A,
                                         const uint32_t *B, int64_t nbatch, int64_t r,
                                         int64_t k, int64_t c, uint64_t p, void *stream);

/* ---------------------------------------------------------------------- */
/* L3: polynomial matrix products                                          */
/* ---------------------------------------------------------------------- */

/* C = A * B.  A: r x k of capacity len1; B: k x c of capacity len2;
 * C: r x c of capacity len1 + len2 - 1 (fully written).
 * Replaces nmod_poly_mat_multiply (flint-extras/src/nmod_poly_mat_extra/mul.c:19-97)
 * and nmod_poly_mat_mul_geometric (mul_geometric.c:121-157).
 * C may not overlap A or B (PMLG_EALIAS); callers that alias use a temporary,
 * as mul.c:42-50 does. */
PMLG_API int pmlg_poly_mat_mul(pmlg_ctx *ctx, uint64_t *C, const uint64_t *A, const uint64_t *B,
                               int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                               uint64_t p, void *stream);

/* res = (A * B mod x^nhi) div x^nlo, res of capacity nhi - nlo (fully written,
 * zero beyond the clamped length).  *out_len (host, may be NULL) receives the
 * clamped length max(0, min(nhi, L1+L2-1) - nlo), L1/L2 the actual max lengths
 * of A/B, as nmod_poly_mat_mulmid (mulmid.c:499-541) computes it; computing it
 * needs a device->host read, so pass NULL to keep the call asynchronous.
 * Replaces nmod_poly_mat_mulmid / _nmod_poly_mat_mulmid (mulmid.c:470-541). */
PMLG_API int pmlg_poly_mat_mulmid(pmlg_ctx *ctx, uint64_t *res, const uint64_t *A,
                                  const uint64_t *B, int64_t r, int64_t k, int64_t c,
                                  int64_t len1, int64_t len2, int64_t nlo, int64_t nhi,
                                  uint64_t p, int64_t *out_len, void *stream);

/* Host-buffer forms of the two products: copies inputs to the device, computes,
 * copies the result back, synchronises `stream`. */
PMLG_API int pmlg_poly_mat_mul_host(pmlg_ctx *ctx, uint64_t *C, const uint64_t *A,
                                    const uint64_t *B, int64_t r, int64_t k, int64_t c,
                                    int64_t len1, int64_t len2, uint64_t p, void *stream);
PMLG_API int pmlg_poly_mat_mulmid_host(pmlg_ctx *ctx, uint64_t *res, const uint64_t *A,
                                       const uint64_t *B, int64_t r, int64_t k, int64_t c,
                                       int64_t len1, int64_t len2, int64_t nlo, int64_t nhi,
                                       uint64_t p, int64_t *out_len, void *stream);

/* A batch of independent products C_i = A_i * B_i with their own shapes,
 * lengths and moduli, computed together.  Device pointers.  Replaces a loop of
 * nmod_poly_mat_multiply calls.  Every job is validated and planned (CRT primes,
 * NTT tables) before anything is launched; the jobs are then spread over the
 * context's batch streams (largest first, onto the least loaded stream, each
 * stream with its own scratch), forked from and joined back to `stream`. */
typedef struct pmlg_polymat_job
{
    int64_t r, k, c, len1, len2;
    uint64_t p;
    const uint64_t *A;
    const uint64_t *B;
    uint64_t *C;            /* capacity len1 + len2 - 1 */
} pmlg_polymat_job;

PMLG_API int pmlg_poly_mat_mul_batch(pmlg_ctx *ctx, const pmlg_polymat_job *jobs, int64_t njobs,
                                     void *stream);

/* ---------------------------------------------------------------------- */
/* L4: approximant bases                                                   */
/* ---------------------------------------------------------------------- */

/* Approximant basis of F (m x n, capacity flen, device) at `order` for the
 * shift `shift` (host, m entries; in: input shift, out: shifted row degree).
 * appbas: device, m x m of capacity appbas_cap >= order + 1 (fully written).
 * *appbas_len (host, may be NULL) receives the max length of appbas.
 * p must be a prime (any word size, 2 <= p < 2^64); m, n <= 1024.  The leaves run on
 * 32-bit residues for p < 2^30 and m, n <= 64, on 64-bit residues otherwise.  The
 * stream is synchronised before return.
 * pmlg_pmbasis replaces nmod_poly_mat_pmbasis
 * (flint-extras/src/nmod_poly_mat_extra/approximant_basis.c:33-69);
 * pmlg_mbasis replaces nmod_poly_mat_mbasis (approximant_basis.c:18-31,
 * nmod_mat_poly_extra/nmod_mat_poly_mbasis.c:116-378). */
PMLG_API int pmlg_pmbasis(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                          const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                          uint64_t p, int64_t *appbas_len, void *stream);
PMLG_API int pmlg_mbasis(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                         const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                         uint64_t p, int64_t *appbas_len, void *stream);
/* Shifted Popov approximant basis (the canonical one): pmbasis with shift s, pmbasis
 * again with shift s - rdeg_s, and the product by the inverse of the second basis'
 * row leading matrix.  Same buffers and conventions as pmlg_pmbasis; shift out: the
 * s-row degree.  Replaces popov_pmbasis
 * (ntl-extras/mat_lzz_pX_extra/src/mat_lzz_pX_pmbasis.cpp:1527-1557), which
 * flint-extras lists as a TODO (nmod_poly_mat_approximant.h:337-348). */
PMLG_API int pmlg_popov_pmbasis(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                                const uint64_t *F, int64_t m, int64_t n, int64_t flen, int64_t order,
                                uint64_t p, int64_t *appbas_len, void *stream);
/* Host-buffer form of pmlg_pmbasis. */
PMLG_API int pmlg_pmbasis_host(pmlg_ctx *ctx, uint64_t *appbas, int64_t appbas_cap, int64_t *shift,
                               const uint64_t *F, int64_t m, int64_t n, int64_t flen,
                               int64_t order, uint64_t p, int64_t *appbas_len, void *stream);

/* Left kernel basis of the m x n polynomial matrix pmat (device, entry stride
 * plen), by the Zhou-Labahn-Storjohann recursion through approximant bases.
 * shift (host, m entries): in = the shift s; out: the s-row degrees of the
 * kernel rows in [0, *nullity).  pivind (host, m entries): out, their s-pivot
 * indices (increasing).  ker: device, m x m of capacity ker_cap; rows
 * [0, *nullity) receive the basis, in s-ordered weak Popov form, the other rows
 * are zero.  *ker_len receives the basis' max length (at least 1); when it is
 * above ker_cap, PMLG_ELEN is returned and nothing is written, so the caller can
 * retry with a larger buffer.  m <= 1024, p any word-size prime.  The stream is
 * synchronised before return.
 * Replaces nmod_poly_mat_kernel_zls_approx
 * (flint-extras/src/nmod_poly_mat_extra/kernel.c:232-480), and
 * nmod_poly_mat_kernel (kernel.c:26-144) with orientation ROW_LOWER. */
PMLG_API int pmlg_kernel_zls(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len,
                             int64_t *pivind, int64_t *shift, const uint64_t *pmat, int64_t m,
                             int64_t n, int64_t plen, uint64_t p, int64_t *nullity, void *stream);
/* nmod_poly_mat_kernel_via_approx (kernel.c:146-227): one approximant basis at the
 * order min(m, n) deg + amp(shift) + deg + 1, whose rows of small shifted degree are
 * the kernel rows.  Same buffers and conventions as pmlg_kernel_zls. */
PMLG_API int pmlg_kernel_via_approx(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len,
                                    int64_t *pivind, int64_t *shift, const uint64_t *pmat, int64_t m,
                                    int64_t n, int64_t plen, uint64_t p, int64_t *nullity, void *stream);
/* nmod_poly_mat_kernel (kernel.c:26-144): the kernel of the r x c matrix pmat (device,
 * entry stride plen) in the given orientation, form at most PMLG_ORD_WEAK_POPOV
 * (PMLG_EUNSUP otherwise, where the reference throws).  Left kernels (PMLG_ROW_*):
 * ker is r x r with the basis in its first *nullity rows; right kernels (PMLG_COL_*):
 * ker is c x c with the basis in its first *nullity columns; the other rows / columns
 * are zero.  shift (host) may be NULL for the default (row or column degrees, zero
 * for zero rows or columns); otherwise it is in/out as in the reference.  pivind
 * (host): the pivot indices.  ker_cap / *ker_len as in pmlg_kernel_zls. */
PMLG_API int pmlg_kernel(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len, int64_t *pivind,
                         int64_t *shift, const uint64_t *pmat, int64_t r, int64_t c, int64_t plen,
                         uint64_t p, int form, int orient, int64_t *nullity, void *stream);
/* Host-buffer form of pmlg_kernel_zls (ker and pmat in host memory). */
PMLG_API int pmlg_kernel_zls_host(pmlg_ctx *ctx, uint64_t *ker, int64_t ker_cap, int64_t *ker_len,
                                  int64_t *pivind, int64_t *shift, const uint64_t *pmat, int64_t m,
                                  int64_t n, int64_t plen, uint64_t p, int64_t *nullity, void *stream);

/* Truncated inverse: S (device, n x n of capacity order + 1) = A^-1 mod x^order for
 * A (device, n x n, entry stride alen), from the approximant basis of [A \\ -I] at
 * order with shift [0, ..., 0, order, ..., order].  *invertible = 1 when A(0) is
 * invertible (S written), 0 otherwise.  n <= 512, p any word-size prime; the stream is
 * synchronised.  Replaces nmod_poly_mat_inv_trunc
 * (flint-extras/src/nmod_poly_mat_extra/nmod_poly_mat_dixon.c:32-80). */
PMLG_API int pmlg_inv_trunc(pmlg_ctx *ctx, uint64_t *S, const uint64_t *A, int64_t n, int64_t alen,
                            int64_t order, uint64_t p, int *invertible, void *stream);
/* Dixon lifting: X (device, n x m of capacity xcap >= ceil(sigma / order) * order)
 * with A X = B mod x^sigma, built one x-adic digit of order coefficients at a time:
 * S = A^-1 B mod x^order, X += x^(l order) S, B <- (B - A S) div x^order.  *ok = 1, or
 * 0 when A(0) is singular.  Replaces nmod_poly_mat_dixon (nmod_poly_mat_dixon.c:92-143). */
PMLG_API int pmlg_dixon(pmlg_ctx *ctx, uint64_t *X, int64_t xcap, const uint64_t *A, const uint64_t *B,
                        int64_t n, int64_t m, int64_t alen, int64_t blen, int64_t order, int64_t sigma,
                        uint64_t p, int *ok, void *stream);

/* Layout conversions (device buffers).  Entry-major (nmod_poly_mat): entry (i, j)
 * holds coefficients at [(i*c + j)*ld, (i*c + j)*ld + len).  Coefficient-major
 * (nmod_mat_poly): coefficient k is the r x c matrix at [k*r*c, (k+1)*r*c).
 * pmlg_poly_mat_to_mat_poly: out (out_cap >= min(order, len) coefficient
 * matrices) receives the coefficients k < min(order, len), zeros past them;
 * *out_len (may be NULL, then nothing synchronises) receives the normalised
 * length, the last nonzero coefficient matrix + 1.  Replaces
 * nmod_mat_poly_set_trunc_from_poly_mat
 * (flint-extras/src/nmod_mat_poly_extra/nmod_mat_poly_set_from.c:31-52).
 * pmlg_mat_poly_to_poly_mat: out (entries of capacity out_cap >= min(order,
 * len)) receives the coefficients k < min(order, len), zeros past them.
 * Replaces nmod_poly_mat_set_trunc_from_mat_poly
 * (flint-extras/src/nmod_poly_mat_extra/nmod_poly_mat_utils.c:185-210). */
PMLG_API int pmlg_poly_mat_to_mat_poly(pmlg_ctx *ctx, uint64_t *out, int64_t out_cap, const uint64_t *in,
                                       int64_t r, int64_t c, int64_t ld, int64_t len, int64_t order,
                                       int64_t *out_len, void *stream);
PMLG_API int pmlg_mat_poly_to_poly_mat(pmlg_ctx *ctx, uint64_t *out, int64_t out_cap, const uint64_t *in,
                                       int64_t r, int64_t c, int64_t len, int64_t order, void *stream);

/* ---------------------------------------------------------------------- */
/* L1: modular dot products and multimodular reduction / CRT               */
/* ---------------------------------------------------------------------- */

/* res[0] (device) = sum_{i<len} v1[i]*v2[i] mod p; entries are arbitrary 64-bit
 * words (not assumed reduced), any 2 <= p < 2^64.
 * Replaces nmod_vec_dot_product_unbalanced
 * (flint-extras/src/nmod_vec_extra/nmod_vec_dot_product.c:136-147) with full
 * 64-bit inputs (the max_bits arguments only bound the accumulator there). */
PMLG_API int pmlg_nmod_vec_dot(pmlg_ctx *ctx, uint64_t *res, const uint64_t *v1,
                               const uint64_t *v2, int64_t len, uint64_t p, void *stream);
/* 32-bit storage, p <= 2^32: replaces _nmod32_vec_dot_split
 * (flint-extras/src/nmod32_vec/dot_split.c:18-47) without its length limit. */
PMLG_API int pmlg_nmod32_vec_dot(pmlg_ctx *ctx, uint32_t *res, const uint32_t *v1,
                                 const uint32_t *v2, int64_t len, uint64_t p, void *stream);
/* mv[i] = sum_{j<len} mat[i*stride + j] * vec[j] mod p, i < nrows, 32-bit storage:
 * replaces _nmod32_vec_mdot_split (flint-extras/src/nmod32_vec/mdot_split.c:17-26). */
PMLG_API int pmlg_nmod32_vec_mdot(pmlg_ctx *ctx, uint32_t *mv, const uint32_t *mat,
                                  const uint32_t *vec, int64_t nrows, int64_t len,
                                  int64_t stride, uint64_t p, void *stream);
/* uv[j] = sum_{i<len} u[i] * v[i*k + j] mod p, j < k (vector-matrix product),
 * 64-bit entries: replaces nmod_vec_dot_product_multi
 * (flint-extras/src/nmod_vec_extra/nmod_vec_dot_product_multi.c:2054), with the
 * rows of v stored contiguously instead of as an array of row pointers. */
PMLG_API int pmlg_nmod_vec_dot_multi(pmlg_ctx *ctx, uint64_t *uv, const uint64_t *u,
                                     const uint64_t *v, int64_t len, int64_t k, uint64_t p,
                                     void *stream);

/* pmlg_nmod_vec_dot_multi without any allocation.  This entry point has no
 * counterpart in the reference; it exists for callers that cannot allocate
 * device memory at the point of the call.  Examples: code that runs under a
 * device-memory budget fixed up front by another allocator, or a pipeline
 * that must not hit the implicit device synchronisation of cudaMalloc/cudaFree
 * in the middle of its work.  It takes no pmlg_ctx.  The partial sums go to a
 * file-scope device array of 65536 x 24 bytes (1.5 MiB), which every GPU that
 * loads the library holds until the process exits.
 * Device pointers; computes the same uv[j] = sum_i u[i] v[i*k + j] mod p as
 * pmlg_nmod_vec_dot_multi, on the current device.
 * - k may be at most 65536; larger k returns PMLG_EUNSUP and nothing runs.
 * - The first call on a device looks up the array's device address
 *   (cudaGetSymbolAddress) with that device current, and keeps it for the rest
 *   of the process.  Make that first call before any stream capture, and do
 *   not use this entry point across a cudaDeviceReset (the kept address would
 *   then be stale).
 * - Every call shares the one array.  Calls that overlap on the GPU (on
 *   different streams, or from different threads) race on it and must be
 *   serialised by the caller.  No state carries over from one call to the
 *   next: every partial sum a call reads, that call wrote first. */
PMLG_API int pmlg_nmod_vec_dot_multi_noalloc(uint64_t *uv, const uint64_t *u, const uint64_t *v,
                                             int64_t len, int64_t k, uint64_t p, void *stream);

/* residues[j*nb + i] = input[i] mod primes[j], j < nprimes <= 6, primes < 2^63:
 * replaces nmod_multimod_CRT_reduce (flint-extras/src/nmod_extra/nmod_multimod_CRT_reduce.c:22). */
PMLG_API int pmlg_multimod_reduce(pmlg_ctx *ctx, uint64_t *residues, const uint64_t *input,
                                  int64_t nb, const uint64_t *primes, int nprimes, void *stream);
/* out[i] = CRT(residues[j*nb + i], j < nprimes) mod p, the CRT value taken in
 * [0, prod primes); primes pairwise coprime, < 2^63:
 * replaces nmod_multimod_CRT_CRT (flint-extras/src/nmod_extra/nmod_multimod_CRT_CRT.c:509). */
PMLG_API int pmlg_multimod_crt(pmlg_ctx *ctx, uint64_t *out, const uint64_t *residues,
                               int64_t nb, const uint64_t *primes, int nprimes, uint64_t p,
                               void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PMLG_H */
