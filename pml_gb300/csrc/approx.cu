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
#include "leaf64.cuh"

#include <cooperative_groups.h>
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
    uint32_t *R;      // [order][m][n]   (general kernel only)
    uint32_t *AB;     // [order+1][m][m] (general kernel only)
    int64_t *shift;   // device, m entries
    int m, n, order;
    uint32_t p, r32, r32q, oneq;
    uint32_t pneg;    // -p^{-1} mod 2^32 (Montgomery reduction)
    uint32_t r2;      // 2^64 mod p (Montgomery conversion)
    int *err;         // device error word: a bounded wait gave up
    unsigned long long *len_out;   // device: a bound on appbas' length (exact unless rows cancel)
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
    __shared__ int s_pl[2], s_rank, s_nn, s_alen, s_grow;

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
    if (tid == 0) s_alen = 1;
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
    if (tid == 0) *a.len_out = (unsigned long long)alen;
}

// ---------------------------------------------------------------------------
// cluster leaf: m <= 64, n <= 32, order <= 32, odd p
// ---------------------------------------------------------------------------
//
// One leaf runs on a cluster of 1 + LC_SL CTAs (one per SM), pipelined over the
// order steps.  CTA 0, the eliminator, holds no slices.  Slice CTA 1+q keeps, in
// its own shared memory, the columns [q*ncm, (q+1)*ncm) of every coefficient of
// appbas and the columns [q*ncn, (q+1)*ncn) of every coefficient of the residual
// R = appbas * F mod x^order, which every row operation keeps up to date (so the
// residual of step s is R[s]).  One cluster barrier phase Q_s per step: CTA 0 has
// published the pivots and X of step s, and the slice CTAs have finished the
// update of step s-1 and pushed the coefficients s+1 and s of their residual
// slices (as they are before step s) into CTA 0's shared memory
// (distributed shared memory stores).
//
// CTA 0, between Q_{s-1} and Q_s: the coefficient s of the residual after step
// s-1 (pivot rows take their coefficient s-1, non-pivot rows add X times the
// pivot rows), permuted and transposed into E = R[s]^T; the elimination of E;
// the pivot inverses and X, while other warps shift the pivot rows' shifts and
// compute the stable shift permutation of step s+1.  The slice CTAs, in the same
// interval: the whole update of step s-1 on their slices.  So the elimination of
// step s, the one chain that cannot be split, runs while the slice CTAs update.
//
// Elimination (CTA 0, its first LC_EW warps): lane j holds row j of E
// (j < n <= 32), warp w holds columns [4w, 4w+4) in registers (LC_EW = 16 warps
// of 4 columns by default); column c's owner warp finds the pivot with a ballot
// and publishes it through shared memory (double-buffered, one barrier per
// column); every warp updates its columns with pivot row values taken by warp
// shuffles.  Updates are division-free,
//   row_j <- (pv * row_j - f_j * row_pl) * 2^-32 mod p   (Montgomery reduction):
// every row operation only scales rows, so the ratios E[pl_b][np_a] / E[pl_b][pc_b]
// at the end are the RREF entries.  Once every row holds a pivot, the remaining
// columns are non-pivots.  X = -RREF restricted to the non-pivot columns, with
// the pivot inverses by Montgomery exponentiation.
//
// Update of step s (slice CTAs): non-pivot rows += X * pivot rows (a whole row
// slice per thread) on appbas' coefficients d < alen and R's coefficients past s;
// pivot rows times x.  The length of appbas grows by one when a pivot row reaches
// its top coefficient (nmod_mat_poly_mbasis.c:306-313): each slice CTA reports it
// into CTA 0, and every slice CTA reads the flags after the next phase.

constexpr int LC_SL = 8;                 // slice CTAs
constexpr int LC_CL = 1 + LC_SL;         // cluster size (a non-portable size, above 8)
constexpr int LC_THREADS = 512;
constexpr int LC_MAXM = 64, LC_MAXN = 32, LC_MAXORD = 32;
#ifndef PMLG_LC_ELIM_WARPS
#define PMLG_LC_ELIM_WARPS 16
#endif
// warps of CTA 0 that run the elimination (each holds 64 / LC_EW columns of E)
constexpr int LC_EW = PMLG_LC_ELIM_WARPS, LC_CPW = LC_MAXM / LC_EW;
static_assert(LC_EW == 4 || LC_EW == 8 || LC_EW == 16, "elimination warps");
static_assert(LC_THREADS == 8 * LC_MAXM, "the permutation takes 8 threads per row");

__device__ __forceinline__ uint32_t redc(uint64_t t, uint32_t p, uint32_t pneg)
{
    // t < p * 2^31: returns t * 2^-32 mod p in [0, p)
    const uint32_t mq = (uint32_t)t * pneg;
    const uint64_t u = t + (uint64_t)mq * p;
    const uint32_t r = (uint32_t)(u >> 32);
    return r >= p ? r - p : r;
}

// b^e mod p by square and multiply in Montgomery form; r2 = 2^64 mod p
__device__ __forceinline__ uint32_t mont_pow(uint32_t b, uint32_t e, uint32_t p, uint32_t pneg, uint32_t r2, uint32_t r1)
{
    uint32_t xm = redc((uint64_t)b * r2, p, pneg);   // b * 2^32 mod p
    uint32_t rm = r1;                               // 1 * 2^32 mod p
    while (e) {
        if (e & 1) rm = redc((uint64_t)rm * xm, p, pneg);
        xm = redc((uint64_t)xm * xm, p, pneg);
        e >>= 1;
    }
    return redc(rm, p, pneg);
}

// split cluster barrier: every thread of every CTA arrives, then waits for the phase
__device__ __forceinline__ void cluster_arrive()
{
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait()
{
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

struct LcShared
{
    uint32_t E[LC_MAXN][LC_MAXM + 1];   // CTA 0: R[s]^T, permuted
    alignas(16) uint32_t X[2][LC_MAXM][LC_MAXN];   // CTA 0: X (nullity x rank) by step parity; slice CTAs: a copy in [0]
    int pivrow[2][LC_MAXM], nprow[2][LC_MAXM];   // likewise
    int info[2][2];                     // CTA 0: rank and nullity by step parity
    int rowidx[LC_MAXM];                // CTA 0: row -> its non-pivot index in the last step, -1 for a pivot row
    int growf[2][LC_SL];                // CTA 0: per-slice growth flags, by step parity
    long long sh[LC_MAXM];              // CTA 0: shifts
    int perm[LC_MAXM];                  // CTA 0: stable shift permutation of the current step
    int pos[LC_MAXM];                   // CTA 0: its inverse (row -> rank)
    uint32_t fbuf[2][32];               // the current column's values, pivot value and
    uint32_t pvbuf[2];                  // pivot lane (double-buffered by column)
    int plbuf[2];
    int pivlane[LC_MAXM], pivcol[LC_MAXM], nonpiv[LC_MAXM];
    uint32_t inv[LC_MAXM];
    alignas(16) uint32_t dpiv[LC_MAXN][LC_MAXN];   // CTA 0: the pivot rows of the last step, gathered
};

// stable shift permutation (rank counting, one thread per row t < m):
// perm[r] = the row of rank r (_find_shift_permutation, nmod_mat_poly_mbasis.c:69-114)
__device__ __forceinline__ void lc_perm(LcShared &S, int m, int t)
{
    if (t < m) {
        const long long v = S.sh[t];
        int r = 0;
        for (int j = 0; j < m; j++) r += (S.sh[j] < v) || (S.sh[j] == v && j < t);
        S.perm[r] = t;
        S.pos[t] = r;
    }
}

// CTA 0, step s: elimination of E = R[s]^T, pivots, X, the shifts of the next step
// and its permutation.  S.perm holds the permutation of step s.  Ends with a block
// barrier.
__device__ void lc_eliminate(LcShared &S, const LeafArgs &a, int s, int tid, int nth)
{
    const int m = a.m, n = a.n;
    const uint32_t p = a.p;
    const int w = tid >> 5, lane = tid & 31;
    int rank = 0, nn = 0;
    if (w < LC_EW) {
        uint32_t x[LC_CPW];
#pragma unroll
        for (int k = 0; k < LC_CPW; k++)
            x[k] = (lane < n && LC_CPW * w + k < m) ? S.E[lane][LC_CPW * w + k] : 0u;
        unsigned used = 0;
        for (int col = 0; col < m; col++) {
            if (rank == n) {
                // every row holds a pivot: the remaining columns are non-pivots
                if (tid == 0) S.nonpiv[nn] = col;
                nn++;
                continue;
            }
            const int buf = col & 1, cw = col / LC_CPW, cl = col % LC_CPW;
            if (w == cw) {
                uint32_t v = x[0];
#pragma unroll
                for (int k = 1; k < LC_CPW; k++)
                    if (cl == k) v = x[k];
                const unsigned cand = __ballot_sync(0xffffffffu, v != 0 && lane < n && !((used >> lane) & 1u));
                const int pl = cand ? __ffs(cand) - 1 : -1;
                S.fbuf[buf][lane] = v;
                if (lane == 0) S.plbuf[buf] = pl;
                if (lane == pl) S.pvbuf[buf] = v;
            }
            if (LC_EW == 16)
                __syncthreads();
            else
                asm volatile("bar.sync 1, %0;" ::"n"(LC_EW * 32) : "memory");
            const int pl = S.plbuf[buf];
            if (pl < 0) {
                if (tid == 0) S.nonpiv[nn] = col;
                nn++;
                continue;
            }
            const uint32_t pv = S.pvbuf[buf];
            const uint32_t f = S.fbuf[buf][lane];
            const uint32_t nf = f ? p - f : 0u;
#pragma unroll
            for (int k = 0; k < LC_CPW; k++) {
                const uint32_t xp = __shfl_sync(0xffffffffu, x[k], pl);
                if (lane != pl) x[k] = redc((uint64_t)x[k] * pv + (uint64_t)nf * xp, p, a.pneg);
            }
            used |= 1u << pl;
            if (tid == 0) { S.pivlane[rank] = pl; S.pivcol[rank] = col; }
            rank++;
        }
#pragma unroll
        for (int k = 0; k < LC_CPW; k++)
            if (lane < n && LC_CPW * w + k < m) S.E[lane][LC_CPW * w + k] = x[k];
    }
    if (tid == 0) S.info[s & 1][0] = rank;
    __syncthreads();
    rank = S.info[s & 1][0];
    const int nullity = m - rank;
    const int par = s & 1;
    if (tid < rank) S.pivrow[par][tid] = S.perm[S.pivcol[tid]];
    if (tid < nullity) S.nprow[par][tid] = S.perm[S.nonpiv[tid]];
    if (tid == 0) S.info[par][1] = nullity;
    __syncthreads();
    // warp 0: pivot inverses; warps 2-3: shifts and permutation of the next step;
    // warps 4-5: row -> non-pivot index
    if (tid < 32) {
        if (tid < rank && nullity > 0)
            S.inv[tid] = mont_pow(S.E[S.pivlane[tid]][S.pivcol[tid]], p - 2, p, a.pneg, a.r2, a.r32);
    } else if (tid >= 64 && tid < 128) {
        const int t = tid - 64;
        if (nullity == 0) {
            if (t < m) S.sh[t] += a.order - s;
        } else {
            if (t < rank) S.sh[S.pivrow[par][t]] += 1;
            asm volatile("bar.sync 2, 64;" ::: "memory");
            lc_perm(S, m, t);
        }
    } else if (tid >= 128 && tid < 192) {
        const int t = tid - 128;
        if (t < m) S.rowidx[t] = -1;
        asm volatile("bar.sync 3, 64;" ::: "memory");
        if (t < nullity) S.rowidx[S.nprow[par][t]] = t;
    }
    __syncthreads();
    if (rank > 0 && nullity > 0) {
        for (int idx = tid; idx < nullity * rank; idx += nth) {
            const int ia = idx / rank, b = idx - ia * rank;
            const uint32_t v = mod64_q((uint64_t)S.E[S.pivlane[b]][S.nonpiv[ia]] * S.inv[b], p,
                                       a.r32, a.r32q, a.oneq);
            S.X[par][ia][b] = v ? p - v : 0u;
        }
    }
    __syncthreads();
}

// slice CTA: the update of step s on its slices (non-pivot rows += X * pivot rows on
// appbas' coefficients d < alen and R's coefficients s < d < order; pivot rows times
// x).  Returns 1 when a pivot row was nonzero at coefficient alen-1 (appbas grows).
__device__ int lc_update(LcShared &S, const LeafArgs &a, uint32_t *AB, uint32_t *R, int sab, int sr, int ncm, int ncn,
                         int cm, int cn, bool vec, int rank, int nullity, int alen, int s, int tid, int nth)
{
    const uint32_t p = a.p;
    const int order = a.order;
    const int nab = nullity * alen;
    const int nr = nullity * (order - s - 1);
    for (int idx = tid; idx < nab + nr; idx += nth) {
        const bool isab = idx < nab;
        const int j2 = isab ? idx : idx - nab;
        const int per = isab ? alen : (order - s - 1);
        const int ia = j2 / per;
        const int d = isab ? j2 - ia * per : s + 1 + (j2 - ia * per);
        const int width = isab ? ncm : ncn, cols = isab ? cm : cn;
        uint32_t *base = isab ? AB + (size_t)d * sab : R + (size_t)d * sr;
        uint32_t *dst = base + S.nprow[0][ia] * width;
        uint64_t acc[8];
        if (vec) {
            // whole rows of 4 or 8 words (columns past `cols` are zero padding)
            const int nq = width >> 2;
#pragma unroll
            for (int h = 0; h < 2; h++)
                if (h < nq) {
                    const uint4 v = *reinterpret_cast<const uint4 *>(dst + 4 * h);
                    acc[4 * h] = v.x; acc[4 * h + 1] = v.y; acc[4 * h + 2] = v.z; acc[4 * h + 3] = v.w;
                } else {
                    acc[4 * h] = acc[4 * h + 1] = acc[4 * h + 2] = acc[4 * h + 3] = 0;
                }
            for (int b0 = 0; b0 < rank; b0 += 8) {
                const int bend = b0 + 8 < rank ? b0 + 8 : rank;
                for (int b = b0; b < bend; b++) {
                    const uint64_t xv = S.X[0][ia][b];
                    const uint32_t *src = base + S.pivrow[0][b] * width;
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        if (h < nq) {
                            const uint4 v = *reinterpret_cast<const uint4 *>(src + 4 * h);
                            acc[4 * h] += xv * v.x; acc[4 * h + 1] += xv * v.y;
                            acc[4 * h + 2] += xv * v.z; acc[4 * h + 3] += xv * v.w;
                        }
                }
#pragma unroll
                for (int u = 0; u < 8; u++) acc[u] = fold(acc[u], a.r32);
            }
#pragma unroll
            for (int h = 0; h < 2; h++)
                if (h < nq) {
                    uint4 v;
                    v.x = mod64_q(acc[4 * h], p, a.r32, a.r32q, a.oneq);
                    v.y = mod64_q(acc[4 * h + 1], p, a.r32, a.r32q, a.oneq);
                    v.z = mod64_q(acc[4 * h + 2], p, a.r32, a.r32q, a.oneq);
                    v.w = mod64_q(acc[4 * h + 3], p, a.r32, a.r32q, a.oneq);
                    *reinterpret_cast<uint4 *>(dst + 4 * h) = v;
                }
            continue;
        }
#pragma unroll
        for (int u = 0; u < 8; u++) acc[u] = (u < cols) ? dst[u] : 0ull;
        for (int b0 = 0; b0 < rank; b0 += 8) {
            const int bend = b0 + 8 < rank ? b0 + 8 : rank;
            for (int b = b0; b < bend; b++) {
                const uint64_t xv = S.X[0][ia][b];
                const uint32_t *src = base + S.pivrow[0][b] * width;
#pragma unroll
                for (int u = 0; u < 8; u++)
                    if (u < cols) acc[u] += xv * src[u];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) acc[u] = fold(acc[u], a.r32);
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (u < cols) dst[u] = mod64_q(acc[u], p, a.r32, a.r32q, a.oneq);
    }
    // growth test on this CTA's columns: a pivot row nonzero at coefficient alen-1
    int grow = 0;
    for (int idx = tid; idx < rank * cm; idx += nth) {
        const int b = idx / cm, col = idx - b * cm;
        if (AB[(size_t)(alen - 1) * sab + S.pivrow[0][b] * ncm + col] != 0) grow = 1;
    }
    grow = __syncthreads_or(grow);
    // pivot rows times x (one coefficient more than the length: it may grow)
    const int nlen = alen + 1 <= order + 1 ? alen + 1 : order + 1;
    for (int idx = tid; idx < rank * (cm + cn); idx += nth) {
        const int b = idx / (cm + cn), col = idx - b * (cm + cn);
        const int row = S.pivrow[0][b];
        if (col < cm) {
            for (int d = nlen - 1; d > 0; d--)
                AB[(size_t)d * sab + row * ncm + col] = AB[(size_t)(d - 1) * sab + row * ncm + col];
            AB[row * ncm + col] = 0;
        } else {
            const int j = col - cm;
            for (int d = order - 1; d > s; d--)
                R[(size_t)d * sr + row * ncn + j] = R[(size_t)(d - 1) * sr + row * ncn + j];
        }
    }
    __syncthreads();
    return grow;
}

__global__ void __launch_bounds__(LC_THREADS)
mbasis_leaf_cluster_kernel(LeafArgs a)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ LcShared S;
    extern __shared__ __align__(16) uint32_t dyn[];
    const int c = (int)cluster.block_rank();
    const int tid = threadIdx.x, nth = blockDim.x;
    const int m = a.m, n = a.n, order = a.order;
    const uint32_t p = a.p;
    const int ncm = (m + LC_SL - 1) / LC_SL, ncn = (n + LC_SL - 1) / LC_SL;
    const int q = c - 1;                                     // slice index of a slice CTA
    const int m0 = q * ncm, n0 = q * ncn;
    const int cm = (c > 0 && m0 < m) ? (m - m0 < ncm ? m - m0 : ncm) : 0;
    const int cn = (c > 0 && n0 < n) ? (n - n0 < ncn ? n - n0 : ncn) : 0;
    // coefficient d of the slices starts at d * sab (appbas) and d * sr (R).  The
    // padding makes threads working on consecutive coefficients of the same row
    // hit distinct banks: 4 words when the slice rows are whole 16-byte vectors
    // (the update then moves rows with 128-bit accesses), 1 word otherwise
    const bool vec = (ncm & 3) == 0 && (ncn & 3) == 0;
    const int sab = m * ncm + (vec ? 4 : 1), sr = m * ncn + (vec ? 4 : 1);
    uint32_t *AB = dyn;                                      // [order+1][m][ncm], padded
    uint32_t *R = dyn + (size_t)(order + 1) * sab;           // [order][m][ncn], padded
    const int64_t fl = a.flen < order ? a.flen : order;

    if (c > 0) {
        for (int idx = tid; idx < order * m * ncn; idx += nth) {
            const int d = idx / (m * ncn), rem = idx - d * m * ncn, i = rem / ncn, jl = rem - i * ncn;
            uint32_t v = 0;
            if (jl < cn && d < fl) v = (uint32_t)a.F[((int64_t)i * n + n0 + jl) * a.ldF + d];
            R[(size_t)d * sr + rem] = v;
        }
        for (int idx = tid; idx < (order + 1) * m * ncm; idx += nth) {
            const int d = idx / (m * ncm), rem = idx - d * m * ncm, i = rem / ncm, il = rem - i * ncm;
            AB[(size_t)d * sab + rem] = (d == 0 && il < cm && i == m0 + il) ? 1u : 0u;
        }
    }
    if (tid < m) S.sh[tid] = a.shift[tid];
    // CTA 0's dynamic shared memory: by step parity, the coefficients s and s-1 of the
    // residual before step s-1, [2][2][m][n]
    uint32_t *D0 = cluster.map_shared_rank(dyn, 0);
    int *growf0 = cluster.map_shared_rank(&S.growf[0][0], 0);
    int alen = 1;              // exact length of appbas (slice CTAs)
    cluster.sync();            // every CTA runs before distributed shared memory is addressed

    if (c > 0) {
        for (int idx = tid; idx < m * cn; idx += nth) {   // R[0] into CTA 0
            const int i = idx / cn, jl = idx - i * cn;
            D0[i * n + n0 + jl] = R[i * ncn + jl];
        }
    } else {
        if (tid < m) lc_perm(S, m, tid);
    }
    cluster_arrive();
    cluster_wait();

    bool pending = false;      // slice CTAs: the update of the previous step is still to apply
    int prank = 0, pnull = 0;  // its rank and nullity
    for (int s = 0; s < order; s++) {
        if (c == 0) {
            // coefficient s of the residual after step s-1, permuted and transposed into E
            const uint32_t *Dc = dyn + (size_t)((s & 1) * 2) * m * n;     // coefficient s
            const uint32_t *Dp = Dc + (size_t)m * n;                       // coefficient s-1
            const int q1 = (s - 1) & 1;
            const int prk = s > 0 ? S.info[q1][0] : 0, pnl = m - prk;
            if (prk == 0) {
                for (int idx = tid; idx < m * n; idx += nth) {
                    const int i = idx / n, j = idx - i * n;
                    S.E[j][S.pos[i]] = Dc[idx];
                }
            } else {
                // pivot rows of step s-1 were multiplied by x: they take their coefficient s-1
                for (int idx = tid; idx < prk * n; idx += nth) {
                    const int b = idx / n, j = idx - b * n, i = S.pivrow[q1][b];
                    S.E[j][S.pos[i]] = Dp[i * n + j];
                }
                // the pivot rows' coefficient s, gathered in pivot order
                for (int idx = tid; idx < prk * n; idx += nth) {
                    const int b = idx / n, j = idx - b * n;
                    S.dpiv[b][j] = Dc[S.pivrow[q1][b] * n + j];
                }
                __syncthreads();
                // non-pivot rows a and a+16 per warp, a lane per column: += X[a][.] * pivot rows,
                // X read 4 entries at a time
                const int w = tid >> 5, lane = tid & 31;
                if (lane < n) {
                    for (int a0 = w; a0 < pnl; a0 += 2 * (LC_THREADS / 32)) {
                        const int a1 = a0 + LC_THREADS / 32;
                        const bool two = a1 < pnl;
                        const int i0 = S.nprow[q1][a0], i1 = two ? S.nprow[q1][a1] : i0;
                        uint64_t acc0 = Dc[i0 * n + lane], acc1 = Dc[i1 * n + lane];
                        uint64_t accb0 = 0, accb1 = 0;
                        for (int b0 = 0; b0 < prk; b0 += 8) {
                            const uint4 x0 = *reinterpret_cast<const uint4 *>(&S.X[q1][a0][b0]);
                            const uint4 x1 = *reinterpret_cast<const uint4 *>(&S.X[q1][two ? a1 : a0][b0]);
                            const uint4 y0 = *reinterpret_cast<const uint4 *>(&S.X[q1][a0][b0 + 4]);
                            const uint4 y1 = *reinterpret_cast<const uint4 *>(&S.X[q1][two ? a1 : a0][b0 + 4]);
                            uint64_t d[8];
#pragma unroll
                            for (int k = 0; k < 8; k++) d[k] = b0 + k < prk ? S.dpiv[b0 + k][lane] : 0u;
                            acc0 += x0.x * d[0] + x0.y * d[1] + x0.z * d[2] + x0.w * d[3];
                            accb0 += y0.x * d[4] + y0.y * d[5] + y0.z * d[6] + y0.w * d[7];
                            acc1 += x1.x * d[0] + x1.y * d[1] + x1.z * d[2] + x1.w * d[3];
                            accb1 += y1.x * d[4] + y1.y * d[5] + y1.z * d[6] + y1.w * d[7];
                            acc0 = fold(acc0, a.r32);
                            acc1 = fold(acc1, a.r32);
                            accb0 = fold(accb0, a.r32);
                            accb1 = fold(accb1, a.r32);
                        }
                        S.E[lane][S.pos[i0]] = mod64_q(acc0 + accb0, p, a.r32, a.r32q, a.oneq);
                        if (two) S.E[lane][S.pos[i1]] = mod64_q(acc1 + accb1, p, a.r32, a.r32q, a.oneq);
                    }
                }
            }
            __syncthreads();
            lc_eliminate(S, a, s, tid, nth);
            cluster_arrive();
            cluster_wait();                              // Q_s
            if (S.info[s & 1][1] == 0) break;
            continue;
        }
        int grow = 0;
        if (pending) grow = lc_update(S, a, AB, R, sab, sr, ncm, ncn, cm, cn, vec, prank, pnull, alen, s - 1, tid, nth);
        if (pending && tid == 0) growf0[((s - 1) & 1) * LC_SL + q] = grow;
        if (s + 1 < order) {
            // coefficients s+1 and s of this slice, as they are before step s, into CTA 0
            uint32_t *Db = D0 + (size_t)(((s + 1) & 1) * 2) * m * n;
            for (int idx = tid; idx < m * cn; idx += nth) {
                const int i = idx / cn, jl = idx - i * cn;
                Db[i * n + n0 + jl] = R[(size_t)(s + 1) * sr + i * ncn + jl];
                Db[(size_t)m * n + i * n + n0 + jl] = R[(size_t)s * sr + i * ncn + jl];
            }
        }
        cluster_arrive();
        cluster_wait();                                  // Q_s
        // the growth of step s-1 in any slice, then rank, pivots and X of step s
        if (pending)
            alen += __syncthreads_or(tid < LC_SL ? growf0[((s - 1) & 1) * LC_SL + tid] : 0);
        const int par = s & 1;
        const int *info0 = cluster.map_shared_rank(&S.info[par][0], 0);
        const int rank = info0[0], nullity = info0[1];
        if (nullity == 0) {
            // appbas = x^(order-s) * appbas (nmod_mat_poly_mbasis.c:221-259)
            const int k = order - s;
            for (int idx = tid; idx < m * ncm; idx += nth) {
                for (int d = alen - 1; d >= 0; d--) AB[((size_t)(d + k)) * sab + idx] = AB[(size_t)d * sab + idx];
                for (int d = 0; d < k; d++) AB[(size_t)d * sab + idx] = 0;
            }
            alen += k;
            pending = false;
            __syncthreads();
            break;
        }
        if (rank > 0) {
            const int *pr0 = cluster.map_shared_rank(&S.pivrow[par][0], 0);
            const int *np0 = cluster.map_shared_rank(&S.nprow[par][0], 0);
            const uint32_t *X0 = cluster.map_shared_rank(&S.X[par][0][0], 0);
            if (tid < rank) S.pivrow[0][tid] = pr0[tid];
            if (tid < nullity) S.nprow[0][tid] = np0[tid];
            for (int idx = tid; idx < nullity * rank; idx += nth) {
                const int ia = idx / rank, b = idx - ia * rank;
                S.X[0][ia][b] = X0[ia * LC_MAXN + b];
            }
            __syncthreads();
        }
        pending = rank > 0;
        prank = rank;
        pnull = nullity;
    }
    if (c > 0 && pending) {
        const int grow = lc_update(S, a, AB, R, sab, sr, ncm, ncn, cm, cn, vec, prank, pnull, alen, order - 1, tid, nth);
        if (tid == 0) growf0[((order - 1) & 1) * LC_SL + q] = grow;
    }
    // the length of appbas: alen, plus one when a pivot row of the last step reached the
    // top coefficient in any slice (pending is the same in every slice CTA)
    cluster.sync();
    if (c == 1) {
        int g = 0;
        if (pending) g = __syncthreads_or(tid < LC_SL ? growf0[((order - 1) & 1) * LC_SL + tid] : 0);
        if (tid == 0) *a.len_out = (unsigned long long)(alen + g <= order + 1 ? alen + g : order + 1);
    }

    // output: columns of this slice, entry-major; coefficients past the length are zero
    if (c > 0) {
        const int olen = alen + 1 <= order + 1 ? alen + 1 : order + 1;
        for (int64_t idx = tid; idx < (int64_t)m * cm * a.ldo; idx += nth) {
            const int64_t e = idx / a.ldo, d = idx - e * a.ldo;
            const int i = (int)(e / cm), il = (int)(e - (int64_t)i * cm);
            a.out[((int64_t)i * m + m0 + il) * a.ldo + d] = d < olen ? (uint64_t)AB[(size_t)d * sab + i * ncm + il] : 0ull;
        }
    }
    if (c == 0 && tid < m) a.shift[tid] = S.sh[tid];
    cluster.sync();   // no CTA leaves while another may still address its shared memory
}

static size_t leaf_cluster_smem(int m, int n, int order)
{
    const int ncm = (m + LC_SL - 1) / LC_SL, ncn = (n + LC_SL - 1) / LC_SL;
    const int pad = ((ncm & 3) == 0 && (ncn & 3) == 0) ? 4 : 1;   // as in the kernel
    const size_t slices = ((size_t)(order + 1) * (m * ncm + pad) + (size_t)order * (m * ncn + pad)) * sizeof(uint32_t);
    const size_t coeffs = (size_t)4 * m * n * sizeof(uint32_t);   // CTA 0: [2][2][m][n]
    return slices > coeffs ? slices : coeffs;
}

// launch (or, with query, the number of co-resident clusters) of the cluster leaf:
// LC_CL CTAs per cluster, a size given at launch because it is above the portable 8
static cudaError_t leaf_cluster_launch(const LeafArgs &a, size_t smem, cudaStream_t st, bool query, int *nclusters)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(LC_CL, 1, 1);
    cfg.blockDim = dim3(LC_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = LC_CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (query) return cudaOccupancyMaxActiveClusters(nclusters, mbasis_leaf_cluster_kernel, &cfg);
    return cudaLaunchKernelEx(&cfg, mbasis_leaf_cluster_kernel, a);
}

// whether a cluster of LC_CL CTAs with the largest leaf's shared memory fits on the
// device (checked once; otherwise the leaves run on the single-CTA kernel)
static bool leaf_cluster_ready()
{
    static int state = 0;   // 0: not checked, 1: ready, -1: unavailable
    if (state == 0) {
        const size_t smax = leaf_cluster_smem(LC_MAXM, LC_MAXN, LC_MAXORD);
        int nc = 0;
        LeafArgs none{};
        state = -1;
        if (cudaFuncSetAttribute(mbasis_leaf_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(mbasis_leaf_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax) ==
                cudaSuccess &&
            leaf_cluster_launch(none, smax, 0, true, &nc) == cudaSuccess && nc >= 1)
            state = 1;
        else
            (void)cudaGetLastError();
    }
    return state == 1;
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

// whether the leaves run on uint64 residues (leaf64.cu): primes from 2^30 up, or more
// than 64 rows or columns
static bool wide_leaf(int64_t m, int64_t n, uint64_t p)
{
    return p >= (1ull << 30) || m > LEAF_MAX || n > LEAF_MAX;
}

// bytes the recursion needs at order o (upper bound)
static size_t pm_arena_bytes(int64_t m, int64_t n, int64_t o, int64_t leaf, bool wide)
{
    if (o <= leaf) {
        if (wide) return leaf64_scratch_bytes((int)m, (int)n, (int)o) + 1024;
        return (size_t)(o * m * n + (o + 1) * m * m) * 4 + 1024;
    }
    const int64_t o1 = o >> 1, o2 = o - o1;
    size_t here = (size_t)(m * m * (o1 + 1) + m * n * o2 + m * m * (o2 + 1)) * 8 + 1024;
    size_t c1 = pm_arena_bytes(m, n, o1, leaf, wide), c2 = pm_arena_bytes(m, n, o2, leaf, wide);
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

// the uint64 leaf: scratch from the arena, one CTA
static int leaf64_run(PmState &S, uint64_t *out, int64_t ldo, const uint64_t *F, int64_t ldF, int64_t flen,
                      int64_t order)
{
    const size_t mark = S.ar.top;
    const int m = (int)S.m, n = (int)S.n, o = (int)order;
    const Leaf64Sizes z = leaf64_sizes(m, n, o);
    Leaf64Args a{};
    a.R = (uint64_t *)S.ar.alloc(z.R);
    a.AB = (uint64_t *)S.ar.alloc(z.AB);
    a.E = z.E ? (uint64_t *)S.ar.alloc(z.E) : nullptr;
    a.X = z.X ? (uint64_t *)S.ar.alloc(z.X) : nullptr;
    a.Xg = a.X;
    a.sh = (long long *)S.ar.alloc(z.sh);
    a.st = (int *)S.ar.alloc(z.st);
    if (!a.R || !a.AB || (z.E && !a.E) || (z.X && !a.X) || !a.sh || !a.st) return PMLG_ENOMEM;
    a.F = F; a.ldF = ldF; a.flen = flen;
    a.out = out; a.ldo = ldo;
    a.shift = S.d_shift;
    a.len_out = S.d_tmp;
    a.m = m; a.n = n; a.order = o;
    leaf64_set_modulus(a, S.p);
    PMLG_TRY(leaf64_launch(S.ctx, a, S.st));
    S.ar.top = mark;
    return PMLG_OK;
}

static int leaf_run(PmState &S, uint64_t *out, int64_t ldo, const uint64_t *F, int64_t ldF, int64_t flen,
                    int64_t order)
{
    if (wide_leaf(S.m, S.n, S.p)) return leaf64_run(S, out, ldo, F, ldF, flen, order);
    const size_t mark = S.ar.top;
    uint32_t *R = (uint32_t *)S.ar.alloc((size_t)(order * S.m * S.n) * 4 + 4);
    uint32_t *AB = (uint32_t *)S.ar.alloc((size_t)((order + 1) * S.m * S.m) * 4);
    if (!R || !AB) return PMLG_ENOMEM;
    LeafArgs a{};
    a.F = F; a.ldF = ldF; a.flen = flen;
    a.out = out; a.ldo = ldo;
    a.R = R; a.AB = AB;
    a.shift = S.d_shift;
    a.err = S.ctx->d_err;
    a.len_out = S.d_tmp;
    a.m = (int)S.m; a.n = (int)S.n; a.order = (int)order;
    a.p = (uint32_t)S.p;
    a.r32 = (uint32_t)((1ull << 32) % S.p);
    a.r32q = h_shoup_q(a.r32, a.p);
    a.oneq = (uint32_t)((1ull << 32) / S.p);
    {
        uint32_t inv = a.p;                       // Newton iteration for p^{-1} mod 2^32 (p odd)
        for (int i = 0; i < 5; i++) inv *= 2u - a.p * inv;
        a.pneg = 0u - inv;
        a.r2 = (uint32_t)h_mulmod(a.r32, a.r32, a.p);
    }
    pmlg_ctx *ctx = S.ctx;
    const bool cluster = (a.p & 1u) && S.m <= LC_MAXM && S.n <= LC_MAXN && order <= LC_MAXORD && leaf_cluster_ready();
    if (cluster) {
        prof_begin(ctx, "mbasis_leaf_cluster", S.st);
        PMLG_CUDA_TRY(leaf_cluster_launch(a, leaf_cluster_smem(a.m, a.n, a.order), S.st, false, nullptr));
        prof_end(ctx, S.st);
    } else {
        prof_begin(ctx, "mbasis_leaf", S.st);
        mbasis_leaf_kernel<<<1, LEAF_THREADS, 0, S.st>>>(a);
        prof_end(ctx, S.st);
    }
    count_launch(ctx);
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
        unsigned long long h = 0;
        PMLG_CUDA_TRY(cudaMemcpyAsync(&h, S.d_tmp, sizeof(h), cudaMemcpyDeviceToHost, S.st));
        PMLG_CUDA_TRY(cudaStreamSynchronize(S.st));
        *len = (int64_t)h;
        return PMLG_OK;
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
        // a bound on the product's length (exact unless the leading coefficients cancel):
        // the products above size their transforms by it, and coefficients past the true
        // length are zero; the entry point measures the exact length once at the end
        *len = j.cnt;
    }
    S.ar.top = mark;
    return PMLG_OK;
}

static int approx_entry(pmlg_ctx *ctx, uint64_t *appbas, int64_t cap, int64_t *shift, const uint64_t *F,
                        int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p, int64_t *out_len,
                        cudaStream_t st, int64_t leaf)
{
    if (!ctx || !shift || m <= 0 || n <= 0 || flen < 0 || order < 0) return PMLG_EINVAL;
    if (cap < order + 1 || !appbas || (flen > 0 && !F)) return PMLG_EINVAL;
    if (m > LEAF64_MAXDIM || n > LEAF64_MAXDIM) {
        set_error(ctx, "approximant bases support m, n <= %d", LEAF64_MAXDIM);
        return PMLG_EUNSUP;
    }
    if (!h_is_prime(p)) {
        set_error(ctx, "approximant bases need a prime modulus");
        return PMLG_EBADMOD;
    }
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t leaf_eff = leaf < 1 ? 1 : leaf;
    const size_t bytes =
        pm_arena_bytes(m, n, order > 0 ? order : 1, leaf_eff, wide_leaf(m, n, p)) + (size_t)m * 8 + 1024;
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
        PMLG_TRY(device_max_length(ctx, appbas, m * m, cap, len, S.d_tmp, &len, st));   // exact
    }
    PMLG_CUDA_TRY(cudaMemcpyAsync(shift, S.d_shift, (size_t)m * 8, cudaMemcpyDeviceToHost, st));
    PMLG_TRY(device_status(ctx, st));
    if (out_len) *out_len = len;
    return PMLG_OK;
}

int pmbasis_device(pmlg_ctx *ctx, uint64_t *appbas, int64_t cap, int64_t *shift, const uint64_t *F,
                   int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p, int64_t *len,
                   cudaStream_t st)
{
    const int64_t leaf = ctx->leaf_order > 0 ? ctx->leaf_order : 32;
    return approx_entry(ctx, appbas, cap, shift, F, m, n, flen, order, p, len, st, leaf);
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
