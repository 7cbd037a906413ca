// leaf64.cu -- the mbasis leaf (nmod_mat_poly_mbasis.c:116-378) on uint64 residues:
// word-size primes p >= 2^30 (up to 2^64) and matrices with more than 64 rows or
// columns, which the 32-bit leaves of approx.cu do not take.
//
// Below 24 rows one CTA of 1024 threads runs all order steps of one leaf, as the 32-bit
// single-CTA leaf does; from 24 rows up the steps run as two launches each (the stepped
// leaf below).  Both keep the residual R = appbas * F mod x^order (coefficient-major)
// and applies every row operation to it, so the residual of step ord is R[ord]
// (coefficient ord of appbas * F is unique: the same steps as recomputing it with
// nmod_mat_poly_mul_coeff, nmod_mat_poly_arith.c:4-41).  Each step:
//   1. the stable sort of (shift[i], i) (_find_shift_permutation, :99-114);
//   2. division-free Gauss-Jordan elimination of the permuted residual's transpose:
//      the column rank profile and, from the ratios E[pl_b][np_a] / E[pl_b][pc_b], the
//      unique RREF that left_nullspace.c:42-102 reads the compact nullspace from;
//   3. non-pivot rows += X * pivot rows, pivot rows times x, shifts of the pivot rows
//      + 1 (:252-359), or appbas *= x^(order-ord) when the nullity is 0 (:221-231).
//
// Arithmetic modulo p: Montgomery reduction with R = 2^64, mul(a, b) = a b 2^-64 mod p
// for a, b < p (p odd).  The elimination step row_j <- pv row_j - f_j row_pl, done as
// mul(pv, row_j) - mul(f_j, row_pl), scales row j by 2^-64 as well: rows are only ever
// scaled by nonzero constants, so the ratios, hence the RREF, are unchanged.  X is kept
// in Montgomery form (X 2^64) so that mul(X_m, v) = X v mod p in the update.  The pivot
// inverses are Fermat powers.  p = 2 (the one even prime) uses bit arithmetic.
#include "leaf64.cuh"

namespace pmlg {

constexpr int L64_THREADS = 1024;
constexpr size_t L64_SMEM_BUDGET = 200 * 1024;

struct M64
{
    uint64_t p, pneg, r2;
    int two;

    // (hi 2^64 + lo) 2^-64 mod p, for hi 2^64 + lo < p 2^64
    __device__ __forceinline__ uint64_t redc(uint64_t lo, uint64_t hi) const
    {
        const uint64_t q = lo * pneg;              // q p = -lo mod 2^64
        const uint64_t qh = __umul64hi(q, p);
        const uint64_t t = hi + qh;                // the low words add up to 0 or 2^64
        bool ovf = t < hi;
        const uint64_t t2 = t + (lo != 0 ? 1ull : 0ull);
        ovf |= t2 < t;
        return (ovf || t2 >= p) ? t2 - p : t2;     // the sum is below 2p
    }
    // a b 2^-64 mod p (a b mod 2 for p = 2)
    __device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) const
    {
        if (two) return a & b;
        return redc(a * b, __umul64hi(a, b));
    }
    // a b mod p
    __device__ __forceinline__ uint64_t mulmod(uint64_t a, uint64_t b) const
    {
        if (two) return a & b;
        return mul(mul(a, b), r2);
    }
    // x 2^64 mod p (x for p = 2)
    __device__ __forceinline__ uint64_t tomont(uint64_t x) const { return two ? x : mul(x, r2); }
    __device__ __forceinline__ uint64_t add(uint64_t a, uint64_t b) const
    {
        const uint64_t s = a + b;
        return (s < a || s >= p) ? s - p : s;
    }
    __device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) const { return a >= b ? a - b : a - b + p; }
    __device__ __forceinline__ uint64_t neg(uint64_t a) const { return a ? p - a : 0; }
    // a^-1 mod p for a != 0, p prime: a^(p-2)
    __device__ uint64_t inv(uint64_t a) const
    {
        if (two) return 1;
        uint64_t xm = tomont(a), rm = tomont(1);
        uint64_t e = p - 2;
        while (e) {
            if (e & 1) rm = mul(rm, xm);
            xm = mul(xm, xm);
            e >>= 1;
        }
        return mul(rm, 1);
    }
};

__host__ __device__ __forceinline__ size_t l64_al(size_t b) { return (b + 15) & ~(size_t)15; }

// dynamic shared memory of the kernel; the kernel carves it in this order
static size_t l64_smem(int m, int n, bool e_sh, bool x_sh)
{
    const size_t mn = m < n ? m : n;
    size_t s = l64_al((size_t)m * 8) + l64_al((size_t)n * 8) + l64_al(mn * 8);
    if (e_sh) s += l64_al((size_t)n * m * 8);
    if (x_sh) s += l64_al((size_t)m * mn * 8);
    s += 6 * l64_al((size_t)m * 4) + l64_al((size_t)n * 4);
    return s;
}

__global__ void __launch_bounds__(L64_THREADS)
mbasis_leaf64_kernel(Leaf64Args a)
{
    extern __shared__ __align__(16) unsigned char l64s[];
    __shared__ int s_pl, s_rank, s_nn, s_alen, s_grow;
    const int tid = threadIdx.x, nth = blockDim.x;
    const int m = a.m, n = a.n, order = a.order;
    const int mn = m < n ? m : n;
    const M64 M{a.p, a.pneg, a.r2, a.two};

    unsigned char *sp = l64s;
    auto take = [&](size_t bytes) {
        unsigned char *r = sp;
        sp += l64_al(bytes);
        return r;
    };
    long long *sh = (long long *)take((size_t)m * 8);
    uint64_t *fac = (uint64_t *)take((size_t)n * 8);
    uint64_t *inv = (uint64_t *)take((size_t)mn * 8);
    uint64_t *E = a.E ? a.E : (uint64_t *)take((size_t)n * m * 8);       // E[j][r], n x m
    uint64_t *X = a.X ? a.X : (uint64_t *)take((size_t)m * mn * 8);      // X[ia][b], nullity x rank
    int *perm = (int *)take((size_t)m * 4);
    int *pivlane = (int *)take((size_t)m * 4);
    int *pivcol = (int *)take((size_t)m * 4);
    int *nonpiv = (int *)take((size_t)m * 4);
    int *pivrow = (int *)take((size_t)m * 4);
    int *nprow = (int *)take((size_t)m * 4);
    int *used = (int *)take((size_t)n * 4);

    const int64_t fl = a.flen < order ? a.flen : order;
    const int64_t mm = (int64_t)m * m, mnn = (int64_t)m * n;
    for (int64_t idx = tid; idx < (int64_t)order * mnn; idx += nth) {
        const int64_t d = idx / mnn, rem = idx - d * mnn;
        a.R[idx] = d < fl ? a.F[rem * a.ldF + d] : 0ull;
    }
    for (int64_t idx = tid; idx < (int64_t)(order + 1) * mm; idx += nth)
        a.AB[idx] = (idx < mm && (idx / m) == (idx % m)) ? 1ull : 0ull;
    for (int t = tid; t < m; t += nth) sh[t] = a.shift[t];
    if (tid == 0) s_alen = 1;
    __syncthreads();

    for (int ord = 0; ord < order; ord++) {
        // 1. stable sort of (shift, index): rank by counting
        for (int t = tid; t < m; t += nth) {
            const long long v = sh[t];
            int r = 0;
            for (int i = 0; i < m; i++) r += (sh[i] < v) || (sh[i] == v && i < t);
            perm[r] = t;
        }
        for (int j = tid; j < n; j += nth) used[j] = 0;
        if (tid == 0) { s_rank = 0; s_nn = 0; }
        __syncthreads();
        for (int64_t idx = tid; idx < mnn; idx += nth) {
            const int r = (int)(idx / n), j = (int)(idx - (int64_t)r * n);
            E[(int64_t)j * m + r] = a.R[((int64_t)ord * m + perm[r]) * n + j];
        }
        __syncthreads();

        // 2. division-free Gauss-Jordan on E (n rows, m columns)
        for (int c = 0; c < m; c++) {
            if (tid < 32) {
                int pl = -1;
                for (int base = 0; base < n && pl < 0; base += 32) {
                    const int l = base + tid;
                    const uint64_t v = (l < n && !used[l]) ? E[(int64_t)l * m + c] : 0ull;
                    const unsigned b = __ballot_sync(0xffffffffu, v != 0);
                    if (b) pl = base + __ffs(b) - 1;
                }
                if (tid == 0) {
                    s_pl = pl;
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
            for (int j = tid; j < n; j += nth) fac[j] = E[(int64_t)j * m + c];
            __syncthreads();
            const int pl = s_pl, rk = s_rank;
            if (pl >= 0) {
                const uint64_t pv = E[(int64_t)pl * m + c];
                for (int64_t idx = tid; idx < mnn; idx += nth) {
                    const int j = (int)(idx / m), cc = (int)(idx - (int64_t)j * m);
                    if (j == pl) continue;
                    E[idx] = M.sub(M.mul(pv, E[idx]), M.mul(fac[j], E[(int64_t)pl * m + cc]));
                }
            }
            __syncthreads();
            if (rk == n) {
                // every row holds a pivot: the remaining columns are non-pivots
                const int nn0 = s_nn;
                for (int t = tid; t < m - 1 - c; t += nth) nonpiv[nn0 + t] = c + 1 + t;
                __syncthreads();
                if (tid == 0) s_nn = nn0 + (m - 1 - c);
                __syncthreads();
                break;
            }
        }
        const int rank = s_rank, nullity = m - rank;
        __syncthreads();   // everyone has read s_rank before it is reset

        if (nullity == 0) {
            // appbas = x^(order-ord) * appbas, shift += order - ord
            const int k = order - ord, alen = s_alen;
            for (int64_t idx = tid; idx < mm; idx += nth) {
                for (int d = alen - 1; d >= 0; d--) a.AB[(int64_t)(d + k) * mm + idx] = a.AB[(int64_t)d * mm + idx];
                for (int d = 0; d < k; d++) a.AB[(int64_t)d * mm + idx] = 0;
            }
            for (int t = tid; t < m; t += nth) sh[t] += k;
            if (tid == 0) s_alen = alen + k;
            __syncthreads();
            break;
        }
        if (rank == 0) continue;   // zero residual: nothing changes

        // compact nullspace, Montgomery form: X[a][b] = -E[pl_b][np_a] / E[pl_b][pc_b] * 2^64
        for (int b = tid; b < rank; b += nth) {
            inv[b] = M.inv(E[(int64_t)pivlane[b] * m + pivcol[b]]);
            pivrow[b] = perm[pivcol[b]];
        }
        for (int ia = tid; ia < nullity; ia += nth) nprow[ia] = perm[nonpiv[ia]];
        __syncthreads();
        for (int64_t idx = tid; idx < (int64_t)nullity * rank; idx += nth) {
            const int ia = (int)(idx / rank), b = (int)(idx - (int64_t)ia * rank);
            const uint64_t x = M.mulmod(E[(int64_t)pivlane[b] * m + nonpiv[ia]], inv[b]);
            X[idx] = M.tomont(M.neg(x));
        }
        for (int b = tid; b < rank; b += nth) sh[pivrow[b]] += 1;
        if (tid == 0) s_grow = 0;
        __syncthreads();

        // 3a. non-pivot rows += X * pivot rows, for appbas (d < alen) and R (ord < d < order)
        const int alen = s_alen;
        const int64_t nab = (int64_t)nullity * alen * m;
        const int64_t nR = (int64_t)nullity * (order - ord - 1) * n;
        for (int64_t idx = tid; idx < nab + nR; idx += nth) {
            uint64_t *base;
            int row, col, width, ia;
            if (idx < nab) {
                ia = (int)(idx / ((int64_t)alen * m));
                const int64_t rem = idx - (int64_t)ia * alen * m;
                const int64_t coef = rem / m;
                col = (int)(rem - coef * m);
                width = m;
                base = a.AB + coef * mm;
            } else {
                const int64_t j2 = idx - nab;
                ia = (int)(j2 / ((int64_t)(order - ord - 1) * n));
                const int64_t rem = j2 - (int64_t)ia * (order - ord - 1) * n;
                const int64_t coef = ord + 1 + rem / n;
                col = (int)(rem % n);
                width = n;
                base = a.R + coef * mnn;
            }
            row = nprow[ia];
            const uint64_t *xr = X + (int64_t)ia * rank;
            uint64_t acc = base[(int64_t)row * width + col];
            for (int b = 0; b < rank; b++) acc = M.add(acc, M.mul(xr[b], base[(int64_t)pivrow[b] * width + col]));
            base[(int64_t)row * width + col] = acc;
        }
        // grow test: a pivot row reaches the top coefficient
        for (int64_t idx = tid; idx < (int64_t)rank * m; idx += nth) {
            const int b = (int)(idx / m), col = (int)(idx - (int64_t)b * m);
            if (a.AB[(int64_t)(alen - 1) * mm + (int64_t)pivrow[b] * m + col] != 0) s_grow = 1;
        }
        __syncthreads();
        const int nlen = alen + (s_grow ? 1 : 0);
        // 3b. pivot rows *= x, in appbas and in R
        for (int64_t idx = tid; idx < (int64_t)rank * (m + n); idx += nth) {
            const int b = (int)(idx / (m + n)), col = (int)(idx - (int64_t)b * (m + n));
            const int row = pivrow[b];
            if (col < m) {
                for (int d = nlen - 1; d > 0; d--)
                    a.AB[(int64_t)d * mm + (int64_t)row * m + col] = a.AB[(int64_t)(d - 1) * mm + (int64_t)row * m + col];
                a.AB[(int64_t)row * m + col] = 0;
            } else {
                const int j = col - m;
                for (int d = order - 1; d > ord; d--)
                    a.R[(int64_t)d * mnn + (int64_t)row * n + j] = a.R[(int64_t)(d - 1) * mnn + (int64_t)row * n + j];
            }
        }
        __syncthreads();
        if (tid == 0) s_alen = nlen;
        __syncthreads();
    }

    // output: entry-major, zero beyond alen
    const int alen = s_alen;
    for (int64_t idx = tid; idx < mm * a.ldo; idx += nth) {
        const int64_t e = idx / a.ldo, d = idx - e * a.ldo;
        a.out[idx] = d < alen ? a.AB[d * mm + e] : 0ull;
    }
    for (int t = tid; t < m; t += nth) a.shift[t] = sh[t];
    if (tid == 0) *a.len_out = (unsigned long long)alen;
}

// ---------------------------------------------------------------------------
// Stepped leaf: the same steps as two launches per order step instead of one CTA for
// the whole leaf.  The elimination (one CTA: the sequential chain of pivots) is
// followed by the row updates of appbas and R spread over the whole GPU; their state
// (shifts, pivot and non-pivot rows, X, rank, the length of appbas) lives in global
// memory between the launches.
//
// Rows are never moved.  Row i of appbas and of R carries an offset off[i], and its
// coefficient d (in appbas and in R alike) sits at the physical coefficient
// d + order - off[i]; multiplying row i by x is off[i] += 1.  The physical
// coefficients below order - off[i] hold the row's (zero) coefficients of negative
// degree, so appbas takes 2 order + 1 physical coefficients and R 2 order.  A step
// whose residual has full rank finishes the leaf (every offset += order - ord) and
// every later launch returns at once.
// ---------------------------------------------------------------------------

// st[]: rank, nullity, alen, grow, finished, mode (0: nothing to do this step,
// 1: update); then the pivot rows, the non-pivot rows and the offsets (m each)
enum { ST_RANK = 0, ST_NUL, ST_ALEN, ST_GROW, ST_FIN, ST_MODE, ST_HDR = 16 };

__global__ void l64s_init(Leaf64Args a)
{
    const int m = a.m, n = a.n, K = a.order;
    const int64_t fl = a.flen < K ? a.flen : K;
    const int64_t mm = (int64_t)m * m, mnn = (int64_t)m * n;
    const int64_t tot_r = (int64_t)2 * K * mnn, tot_a = (int64_t)(2 * K + 1) * mm;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < tot_r + tot_a + m;
         idx += (int64_t)gridDim.x * blockDim.x) {
        if (idx < tot_r) {
            const int64_t ph = idx / mnn, rem = idx - ph * mnn, d = ph - K;
            a.R[idx] = (d >= 0 && d < fl) ? a.F[rem * a.ldF + d] : 0ull;
        } else if (idx < tot_r + tot_a) {
            const int64_t i = idx - tot_r, ph = i / mm, e = i - ph * mm;
            a.AB[i] = (ph == K && (e / m) == (e % m)) ? 1ull : 0ull;
        } else {
            const int t = (int)(idx - tot_r - tot_a);
            a.sh[t] = a.shift[t];
            a.st[ST_HDR + 2 * m + t] = 0;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < ST_HDR) a.st[threadIdx.x] = threadIdx.x == ST_ALEN ? 1 : 0;
}

// (a b - c d) 2^-64 mod p for a, b, c, d < p: one reduction of a b + (p - c) d, which is
// below 2 p^2 <= p 2^64 for p < 2^63; two reductions above
__device__ __forceinline__ uint64_t l64_fms(const M64 &M, uint64_t a, uint64_t b, uint64_t c, uint64_t d)
{
    if (M.two) return (a & b) ^ (c & d);
    if (M.p >> 63) return M.sub(M.mul(a, b), M.mul(c, d));
    const uint64_t c2 = M.p - c;
    const uint64_t l1 = a * b, h1 = __umul64hi(a, b);
    const uint64_t l2 = c2 * d, h2 = __umul64hi(c2, d);
    const uint64_t lo = l1 + l2;
    return M.redc(lo, h1 + h2 + (lo < l1 ? 1ull : 0ull));
}

// shared memory of the elimination CTA: shifts, pivot diagonals, inverses, E (when it
// fits), then the integer arrays (as l64_smem with X in global memory)
__global__ void __launch_bounds__(L64_THREADS)
l64s_elim(Leaf64Args a, int ord)
{
    extern __shared__ __align__(16) unsigned char l64s[];
    __shared__ int s_stop;
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31;
    const int m = a.m, n = a.n, K = a.order;
    const int mn = m < n ? m : n;
    const int ldE = m | 1;   // odd row stride: a column of E spreads over the banks
    const M64 M{a.p, a.pneg, a.r2, a.two};
    int *st = a.st;
    if (tid == 0) {
        s_stop = st[ST_FIN];
        if (s_stop) {
            st[ST_MODE] = 0;
        } else {
            st[ST_ALEN] += st[ST_GROW];   // the previous step's growth
            st[ST_GROW] = 0;
        }
    }
    unsigned char *sp = l64s;
    auto take = [&](size_t bytes) {
        unsigned char *r = sp;
        sp += l64_al(bytes);
        return r;
    };
    long long *sh = (long long *)take((size_t)m * 8);
    uint64_t *diag = (uint64_t *)take((size_t)n * 8);   // pivot b's entry E[pl_b][pc_b]
    uint64_t *inv = (uint64_t *)take((size_t)mn * 8);
    uint64_t *E = a.E ? a.E : (uint64_t *)take((size_t)n * ldE * 8);
    int *perm = (int *)take((size_t)m * 4);
    int *pivlane = (int *)take((size_t)m * 4);
    int *pivcol = (int *)take((size_t)m * 4);
    int *nonpiv = (int *)take((size_t)m * 4);
    int *soff = (int *)take((size_t)m * 4);
    (void)take((size_t)m * 4);
    (void)take((size_t)n * 4);
    int *pivrow = st + ST_HDR, *nprow = st + ST_HDR + m, *off = st + ST_HDR + 2 * m;
    const int mnn = m * n;
    const int64_t plane = (int64_t)mnn;

    for (int t = tid; t < m; t += nth) { sh[t] = a.sh[t]; soff[t] = off[t]; }
    __syncthreads();
    if (s_stop) return;
    // 1. stable sort of (shift, index): rank by counting
    for (int t = tid; t < m; t += nth) {
        const long long v = sh[t];
        int r = 0;
        for (int i = 0; i < m; i++) r += (sh[i] < v) || (sh[i] == v && i < t);
        perm[r] = t;
    }
    __syncthreads();
    for (int idx = tid; idx < mnn; idx += nth) {
        const int r = idx / n, j = idx - r * n, row = perm[r];
        E[j * ldE + r] = a.R[(int64_t)(ord + K - soff[row]) * plane + row * n + j];
    }
    __syncthreads();
    // 2. division-free Gauss-Jordan on E (n rows, m columns).  Every warp finds the pivot
    // itself (the same one), so a pivot column costs one barrier.  Only the entries read
    // later are computed: the columns right of c and the non-pivot columns left of it.
    // The other entries of a pivot column are 0, its diagonal is scaled by every later
    // pivot value.
    unsigned usedbits = 0;   // bit k of lane l: row 32 k + l holds a pivot
    int rk = 0, nn = 0;
    // up to 64 columns and 32 rows: one thread per column and two rows of E
    const bool small = m <= 64 && n <= 32 && nth == 1024;
    const int mycol = tid & 63, myrow = tid >> 6;
    bool mynp = false;   // this thread's column is a non-pivot column
    for (int c = 0; c < m; c++) {
        int pl = -1;
        for (int k = 0, base = 0; base < n && pl < 0; k++, base += 32) {
            const int l = base + lane;
            const uint64_t v = (l < n && !((usedbits >> k) & 1u)) ? E[l * ldE + c] : 0ull;
            const unsigned b = __ballot_sync(0xffffffffu, v != 0);
            if (b) pl = base + __ffs(b) - 1;
        }
        if (pl < 0) {
            if (tid == 0) nonpiv[nn] = c;
            if (mycol == c) mynp = true;
            nn++;
            __syncthreads();
            continue;
        }
        if ((pl & 31) == lane) usedbits |= 1u << (pl >> 5);
        const uint64_t pv = E[pl * ldE + c];
        for (int b = tid; b < rk; b += nth) diag[b] = M.mul(pv, diag[b]);
        if (tid == 0) { pivlane[rk] = pl; pivcol[rk] = c; diag[rk] = pv; }
        rk++;
        const int W = nn + (m - 1 - c);   // columns updated
        const int tot = (n - 1) * W;
        if (small) {
            // thread = (column, rows r and r + 16): the same entries as below, without
            // the index arithmetic
            if (mycol < m && mycol != c && (mycol > c || mynp)) {
                const uint64_t er = E[pl * ldE + mycol];
                for (int j = myrow; j < n; j += 16) {
                    if (j == pl) continue;
                    uint64_t *e = E + j * ldE + mycol;
                    *e = l64_fms(M, pv, *e, E[j * ldE + c], er);
                }
            }
        } else if (tot > 0) {
            int jj = tid / W, w = tid - jj * W;
            const int dj = nth / W, dw = nth - dj * W;
            const uint64_t *er = E + pl * ldE;
            for (int idx = tid; idx < tot; idx += nth) {
                const int j = jj + (jj >= pl ? 1 : 0);
                const int cc = w < nn ? nonpiv[w] : c + 1 + (w - nn);
                uint64_t *e = E + j * ldE + cc;
                *e = l64_fms(M, pv, *e, E[j * ldE + c], er[cc]);
                jj += dj;
                w += dw;
                if (w >= W) { w -= W; jj++; }
            }
        }
        __syncthreads();
        if (rk == n) {
            for (int t = tid; t < m - 1 - c; t += nth) nonpiv[nn + t] = c + 1 + t;
            nn += m - 1 - c;
            break;
        }
    }
    __syncthreads();
    const int rank = rk, nullity = m - rank;
    if (nullity == 0) {
        // appbas = x^(order-ord) * appbas, shift += order - ord; done
        const int k = K - ord;
        for (int t = tid; t < m; t += nth) { a.sh[t] = sh[t] + k; off[t] = soff[t] + k; }
        if (tid == 0) { st[ST_ALEN] += k; st[ST_FIN] = 1; st[ST_MODE] = 0; }
        return;
    }
    if (rank == 0) {
        if (tid == 0) st[ST_MODE] = 0;   // zero residual: nothing changes
        return;
    }
    for (int b = tid; b < rank; b += nth) {
        inv[b] = M.inv(diag[b]);
        pivrow[b] = perm[pivcol[b]];
    }
    for (int ia = tid; ia < nullity; ia += nth) nprow[ia] = perm[nonpiv[ia]];
    __syncthreads();
    for (int idx = tid; idx < nullity * rank; idx += nth) {
        const int ia = idx / rank, b = idx - ia * rank;
        const uint64_t x = M.mulmod(E[pivlane[b] * ldE + nonpiv[ia]], inv[b]);
        a.Xg[idx] = M.tomont(M.neg(x));
    }
    // the pivot rows: shift + 1, times x
    for (int b = tid; b < rank; b += nth) {
        const int row = perm[pivcol[b]];
        a.sh[row] = sh[row] + 1;
        off[row] = soff[row] + 1;
    }
    if (tid == 0) { st[ST_RANK] = rank; st[ST_NUL] = nullity; st[ST_MODE] = 1; }
}

// non-pivot rows += X * pivot rows (appbas d < alen, R ord < d < order), the pivot rows
// read at their offsets before this step's x; the growth test on the pivot rows'
// coefficient alen - 1.  Dynamic shared memory: 2 rank ints.
__global__ void l64s_update(Leaf64Args a, int ord)
{
    extern __shared__ int l64u[];
    const int *st = a.st;
    if (st[ST_MODE] != 1) return;
    const M64 M{a.p, a.pneg, a.r2, a.two};
    const int m = a.m, n = a.n, K = a.order;
    const int64_t mm = (int64_t)m * m, mnn = (int64_t)m * n;
    const int alen = st[ST_ALEN], rank = st[ST_RANK], nullity = st[ST_NUL];
    const int *pivrow = st + ST_HDR, *nprow = st + ST_HDR + m, *off = st + ST_HDR + 2 * m;
    int *prow = l64u, *poff = l64u + rank;   // pivot rows, their offsets before the step
    for (int b = threadIdx.x; b < rank; b += blockDim.x) {
        prow[b] = pivrow[b];
        poff[b] = off[pivrow[b]] - 1;
    }
    __syncthreads();
    const int64_t g0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
    const int64_t per_a = (int64_t)alen * m, per_r = (int64_t)(K - ord - 1) * n;
    const int64_t nab = (int64_t)nullity * per_a, nR = (int64_t)nullity * per_r;
    for (int64_t idx = g0; idx < nab + nR; idx += gs) {
        uint64_t *base;
        int64_t pl, d;
        int col, width, ia;
        if (idx < nab) {
            ia = (int)(idx / per_a);
            const int64_t rem = idx - (int64_t)ia * per_a;
            d = rem / m;
            col = (int)(rem - d * m);
            width = m;
            base = a.AB;
            pl = mm;
        } else {
            const int64_t j2 = idx - nab;
            ia = (int)(j2 / per_r);
            const int64_t rem = j2 - (int64_t)ia * per_r;
            d = ord + 1 + rem / n;
            col = (int)(rem % n);
            width = n;
            base = a.R;
            pl = mnn;
        }
        const int row = nprow[ia];
        const uint64_t *xr = a.Xg + (int64_t)ia * rank;
        uint64_t *dst = base + (d + K - off[row]) * pl + (int64_t)row * width + col;
        const uint64_t *src = base + (d + K) * pl + col;
        uint64_t acc = *dst;
        // eight pivot rows at a time: their loads are issued together instead of one
        // global-memory latency per pivot row
        int b = 0;
        for (; b + 8 <= rank; b += 8) {
            uint64_t xv[8], pv[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                xv[u] = xr[b + u];
                pv[u] = src[(int64_t)prow[b + u] * width - poff[b + u] * pl];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) acc = M.add(acc, M.mul(xv[u], pv[u]));
        }
        for (; b < rank; b++)
            acc = M.add(acc, M.mul(xr[b], src[(int64_t)prow[b] * width - poff[b] * pl]));
        *dst = acc;
    }
    int grow = 0;
    for (int64_t idx = g0; idx < (int64_t)rank * m; idx += gs) {
        const int b = (int)(idx / m), col = (int)(idx - (int64_t)b * m);
        if (a.AB[(int64_t)(alen - 1 + K - poff[b]) * mm + (int64_t)prow[b] * m + col] != 0) grow = 1;
    }
    if (__syncthreads_or(grow) && threadIdx.x == 0) atomicOr(a.st + ST_GROW, 1);
}

// appbas out (entry-major, zero past its length), the shifts and the length
__global__ void l64s_final(Leaf64Args a)
{
    const int m = a.m, K = a.order;
    const int64_t mm = (int64_t)m * m;
    const int alen = a.st[ST_ALEN] + a.st[ST_GROW];
    const int *off = a.st + ST_HDR + 2 * m;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < mm * a.ldo;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx / a.ldo, d = idx - e * a.ldo;
        a.out[idx] = d < alen ? a.AB[(d + K - off[e / m]) * mm + e] : 0ull;
    }
    if (blockIdx.x == 0) {
        for (int t = threadIdx.x; t < m; t += blockDim.x) a.shift[t] = a.sh[t];
        if (threadIdx.x == 0) *a.len_out = (unsigned long long)alen;
    }
}

// the stepped leaf pays two launches per order step; it takes over from the one-CTA
// kernel when the rows are many enough that the updates outweigh the launches
static bool l64_stepped(int m, int n)
{
    return m >= 24 || (int64_t)m * (m + n) >= 1536;
}

static size_t l64_round(size_t b) { return (b + 255) & ~(size_t)255; }

Leaf64Sizes leaf64_sizes(int m, int n, int order)
{
    const size_t mn = m < n ? m : n;
    Leaf64Sizes z{};
    z.stepped = l64_stepped(m, n);
    const bool e_sh = l64_smem(z.stepped ? m + 1 : m, n, true, false) <= L64_SMEM_BUDGET;
    const bool x_sh = !z.stepped && l64_smem(m, n, e_sh, true) <= L64_SMEM_BUDGET;
    const size_t cr = z.stepped ? 2 * (size_t)order : (size_t)order;
    const size_t ca = z.stepped ? 2 * (size_t)order + 1 : (size_t)order + 1;
    z.R = cr * m * n * 8 + 8;
    z.AB = ca * m * m * 8;
    z.E = e_sh ? 0 : (size_t)n * (m + 1) * 8;
    z.X = x_sh ? 0 : (size_t)m * mn * 8;
    z.sh = (size_t)m * 8;
    z.st = (size_t)(ST_HDR + 3 * m) * 4;
    return z;
}

size_t leaf64_scratch_bytes(int m, int n, int order)
{
    const Leaf64Sizes z = leaf64_sizes(m, n, order);
    return l64_round(z.R) + l64_round(z.AB) + l64_round(z.E) + l64_round(z.X) + l64_round(z.sh) + l64_round(z.st);
}

void leaf64_set_modulus(Leaf64Args &a, uint64_t p)
{
    a.p = p;
    a.two = p == 2;
    if (p & 1) {
        uint64_t inv = p;                       // p^-1 mod 2^64 by Newton (correct to 3 bits at start)
        for (int i = 0; i < 6; i++) inv *= 2 - p * inv;
        a.pneg = 0 - inv;
        a.r1 = (0 - p) % p;                     // 2^64 mod p
        a.r2 = h_mulmod(a.r1, a.r1, p);         // 2^128 mod p
    } else {
        a.pneg = 0;
        a.r1 = 0;
        a.r2 = 0;
    }
}

int leaf64_launch(pmlg_ctx *ctx, const Leaf64Args &a, cudaStream_t st)
{
    if (l64_stepped(a.m, a.n)) {
        const int m = a.m, n = a.n, order = a.order;
        const size_t smem = l64_smem(m + 1, n, a.E == nullptr, false);
        PMLG_CUDA_TRY(cudaFuncSetAttribute(l64s_elim, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        auto grid_for = [&](int64_t work) {
            int64_t g = (work + 255) / 256;
            const int64_t cap = (int64_t)ctx->sm_count * 8;
            return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
        };
        const int64_t mm = (int64_t)m * m, mnn = (int64_t)m * n;
        const size_t usmem = (size_t)2 * (m < n ? m : n) * sizeof(int);
        prof_begin(ctx, "mbasis_leaf64_init", st);
        l64s_init<<<grid_for((int64_t)2 * order * mnn + (int64_t)(2 * order + 1) * mm + m), 256, 0, st>>>(a);
        prof_end(ctx, st);
        const unsigned gu = grid_for((int64_t)m * (m * (int64_t)(order + 1) + n * (int64_t)order));
        for (int ord = 0; ord < order; ord++) {
            prof_begin(ctx, "mbasis_leaf64_elim", st);
            l64s_elim<<<1, L64_THREADS, smem, st>>>(a, ord);
            prof_end(ctx, st);
            prof_begin(ctx, "mbasis_leaf64_update", st);
            l64s_update<<<gu, 256, usmem, st>>>(a, ord);
            prof_end(ctx, st);
        }
        prof_begin(ctx, "mbasis_leaf64_final", st);
        l64s_final<<<grid_for(mm * a.ldo), 256, 0, st>>>(a);
        prof_end(ctx, st);
        count_launch(ctx, (unsigned)(2 * order + 2));
        PMLG_CUDA_TRY(cudaGetLastError());
        return PMLG_OK;
    }
    const size_t smem = l64_smem(a.m, a.n, a.E == nullptr, a.X == nullptr);
    PMLG_CUDA_TRY(cudaFuncSetAttribute(mbasis_leaf64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    prof_begin(ctx, "mbasis_leaf64", st);
    mbasis_leaf64_kernel<<<1, L64_THREADS, smem, st>>>(a);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

}  // namespace pmlg
