/*
 * pmlg_oracle.c -- CPU restatement of PML's evaluation/interpolation hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the timed CPU
 * baseline.  Nothing in the product library links or calls this file.
 * See pmlg_oracle.h for the parity status and the layouts.
 */
#include "pmlg_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* generator                                                           */
/* ------------------------------------------------------------------ */

uint64_t orc_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

/* uniform in [0,p): draw 64-bit words, reject those at or above the largest
 * multiple of p, reduce the rest */
static uint64_t rand_below(uint64_t *st, uint64_t p)
{
    const uint64_t lim = UINT64_MAX - (UINT64_MAX % p + 1) % p; /* keep x <= lim */
    for (;;)
    {
        uint64_t x = orc_splitmix64(st);
        if (x <= lim)
            return x % p;
    }
}

void orc_rand_vec(uint64_t *v, int64_t n, uint64_t p, uint64_t seed)
{
    uint64_t st = seed;
    for (int64_t i = 0; i < n; i++)
        v[i] = rand_below(&st, p);
}

void orc_rand_vec_u32(uint32_t *v, int64_t n, uint64_t p, uint64_t seed)
{
    uint64_t st = seed;
    for (int64_t i = 0; i < n; i++)
        v[i] = (uint32_t) rand_below(&st, p);
}

/* ------------------------------------------------------------------ */
/* scalars                                                             */
/* ------------------------------------------------------------------ */

uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t p)
{
    return (uint64_t) (((u128) a * b) % p);
}

static inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t p)
{
    uint64_t s = a + b;
    if (s < a || s >= p)
        s -= p;
    return s;
}

static inline uint64_t submod(uint64_t a, uint64_t b, uint64_t p)
{
    return (a >= b) ? a - b : a + (p - b);
}

uint64_t orc_powmod(uint64_t a, uint64_t e, uint64_t p)
{
    uint64_t r = 1 % p;
    a %= p;
    while (e)
    {
        if (e & 1)
            r = orc_mulmod(r, a, p);
        a = orc_mulmod(a, a, p);
        e >>= 1;
    }
    return r;
}

uint64_t orc_invmod(uint64_t a, uint64_t p)
{
    /* extended Euclid on signed 128-bit values */
    __int128 t = 0, nt = 1, r = p, nr = a % p;
    while (nr != 0)
    {
        __int128 q = r / nr, tmp;
        tmp = t - q * nt; t = nt; nt = tmp;
        tmp = r - q * nr; r = nr; nr = tmp;
    }
    if (r != 1)
        return 0;
    if (t < 0)
        t += p;
    return (uint64_t) t;
}

int orc_is_prime(uint64_t n)
{
    if (n < 2)
        return 0;
    static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (int i = 0; i < 12; i++)
    {
        if (n == small[i])
            return 1;
        if (n % small[i] == 0)
            return 0;
    }
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) { d >>= 1; s++; }
    /* these 12 bases are a deterministic Miller-Rabin set for n < 2^64 */
    for (int i = 0; i < 12; i++)
    {
        uint64_t x = orc_powmod(small[i], d, n);
        if (x == 1 || x == n - 1)
            continue;
        int comp = 1;
        for (int r = 1; r < s; r++)
        {
            x = orc_mulmod(x, x, n);
            if (x == n - 1) { comp = 0; break; }
        }
        if (comp)
            return 0;
    }
    return 1;
}

uint64_t orc_rand_prime(int bits, uint64_t seed)
{
    uint64_t st = seed;
    for (;;)
    {
        uint64_t x = orc_splitmix64(&st);
        x &= (bits >= 64) ? UINT64_MAX : ((1ULL << bits) - 1);
        x |= 1ULL << (bits - 1);
        x |= 1;
        if (orc_is_prime(x))
            return x;
    }
}

uint64_t orc_find_root(uint64_t n, uint64_t p)
{
    for (uint64_t q = 2; q < p; q++)
    {
        uint64_t k = 1, qk = q;
        while (qk != 1 && k < n)
        {
            qk = orc_mulmod(qk, q, p);
            k++;
        }
        if (qk != 1)
            return q;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* matrices                                                            */
/* ------------------------------------------------------------------ */

/* dot product of k terms a[i*sa] * b[i*sb] mod p, all entries < p */
static uint64_t dot_strided(const uint64_t *a, int64_t sa, const uint64_t *b, int64_t sb,
                            int64_t k, uint64_t p)
{
    if (p <= (1ULL << 32))
    {
        /* products < 2^64: a 128-bit accumulator cannot overflow for k < 2^64 */
        u128 acc = 0;
        for (int64_t i = 0; i < k; i++)
            acc += (u128) (a[i * sa] * b[i * sb]);
        return (uint64_t) (acc % p);
    }
    uint64_t acc = 0;
    for (int64_t i = 0; i < k; i++)
        acc = addmod(acc, orc_mulmod(a[i * sa], b[i * sb], p), p);
    return acc;
}

void orc_nmod_mat_mul(uint64_t *C, const uint64_t *A, const uint64_t *B,
                      int64_t r, int64_t k, int64_t c, uint64_t p)
{
    for (int64_t i = 0; i < r; i++)
        for (int64_t j = 0; j < c; j++)
            C[i * c + j] = dot_strided(A + i * k, 1, B + j, c, k, p);
}

void orc_nmod_mat_mul_batch_u32(uint32_t *C, const uint32_t *A, const uint32_t *B,
                                int64_t nbatch, int64_t r, int64_t k, int64_t c,
                                uint64_t p, int nthreads)
{
    (void) nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int64_t b = 0; b < nbatch; b++)
    {
        const uint32_t *Ab = A + b * r * k;
        const uint32_t *Bb = B + b * k * c;
        uint32_t *Cb = C + b * r * c;
        for (int64_t i = 0; i < r; i++)
            for (int64_t j = 0; j < c; j++)
            {
                u128 acc = 0;
                for (int64_t l = 0; l < k; l++)
                    acc += (uint64_t) Ab[i * k + l] * Bb[l * c + j];
                Cb[i * c + j] = (uint32_t) (acc % p);
            }
    }
}

int64_t orc_nmod_mat_rref(uint64_t *A, int64_t r, int64_t c, uint64_t p)
{
    int64_t rank = 0;
    for (int64_t col = 0; col < c && rank < r; col++)
    {
        int64_t piv = -1;
        for (int64_t i = rank; i < r; i++)
            if (A[i * c + col] % p != 0) { piv = i; break; }
        if (piv < 0)
            continue;
        if (piv != rank)
            for (int64_t j = 0; j < c; j++)
            {
                uint64_t t = A[piv * c + j];
                A[piv * c + j] = A[rank * c + j];
                A[rank * c + j] = t;
            }
        uint64_t inv = orc_invmod(A[rank * c + col], p);
        for (int64_t j = 0; j < c; j++)
            A[rank * c + j] = orc_mulmod(A[rank * c + j], inv, p);
        for (int64_t i = 0; i < r; i++)
        {
            if (i == rank)
                continue;
            uint64_t f = A[i * c + col];
            if (f == 0)
                continue;
            for (int64_t j = 0; j < c; j++)
                A[i * c + j] = submod(A[i * c + j], orc_mulmod(f, A[rank * c + j], p), p);
        }
        rank++;
    }
    return rank;
}

int64_t orc_nmod_mat_rank(const uint64_t *A, int64_t r, int64_t c, uint64_t p)
{
    uint64_t *T = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (r * c + 1));
    memcpy(T, A, sizeof(uint64_t) * (size_t) (r * c));
    int64_t rk = orc_nmod_mat_rref(T, r, c, p);
    free(T);
    return rk;
}

/*
 * Left nullspace in compact form, restating left_nullspace.c:42-102 on top of
 * FLINT's nmod_mat_nullspace: the kernel basis of At = A^T is built from the
 * (unique) RREF R of At, one column per non-pivot column f of R, with 1 at f
 * and -R[j][f] at pivot column p_j.  Hence pivots of R = row rank profile of A
 * (perm[0..rank)), non-pivots = complement (perm[rank..m)), and the compact
 * nullspace is X[i][j] = -R[j][nonpivot_i].
 */
int64_t orc_left_nullspace_compact(uint64_t *X, int64_t *perm,
                                   const uint64_t *A, int64_t m, int64_t n, uint64_t p)
{
    uint64_t *R = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (n * m + 1));
    for (int64_t i = 0; i < m; i++)
        for (int64_t j = 0; j < n; j++)
            R[j * m + i] = A[i * n + j];
    const int64_t rank = orc_nmod_mat_rref(R, n, m, p);
    const int64_t nullity = m - rank;
    /* pivot columns of R, increasing */
    int64_t np = 0, nn = 0;
    int64_t *piv = (int64_t *) malloc(sizeof(int64_t) * (size_t) (m + 1));
    int64_t *nonpiv = (int64_t *) malloc(sizeof(int64_t) * (size_t) (m + 1));
    {
        int64_t row = 0;
        for (int64_t col = 0; col < m; col++)
        {
            if (row < rank && R[row * m + col] != 0)
            {
                piv[np++] = col;
                row++;
            }
            else
                nonpiv[nn++] = col;
        }
    }
    if (nullity == 0)
    {
        for (int64_t i = 0; i < m; i++)
            perm[i] = i;
    }
    else
    {
        for (int64_t j = 0; j < rank; j++)
            perm[j] = piv[j];
        for (int64_t i = 0; i < nullity; i++)
            perm[rank + i] = nonpiv[i];
        for (int64_t i = 0; i < nullity; i++)
            for (int64_t j = 0; j < rank; j++)
            {
                uint64_t v = R[j * m + nonpiv[i]];
                X[i * rank + j] = v ? p - v : 0;
            }
    }
    free(R);
    free(piv);
    free(nonpiv);
    return nullity;
}

/* ------------------------------------------------------------------ */
/* polynomial matrices                                                 */
/* ------------------------------------------------------------------ */

int64_t orc_pm_max_length(const uint64_t *P, int64_t r, int64_t c, int64_t cap)
{
    int64_t L = 0;
    for (int64_t e = 0; e < r * c; e++)
    {
        int64_t l = cap;
        while (l > L && P[e * cap + l - 1] == 0)
            l--;
        if (l > L)
            L = l;
    }
    return L;
}

/* coefficient range [lo, hi) of the product entry sum_l A_il * B_lj */
static void pm_mul_range(uint64_t *C, int64_t ccap, const uint64_t *A, const uint64_t *B,
                         int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                         int64_t lo, int64_t hi, uint64_t p, int nthreads)
{
    (void) nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) collapse(2) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int64_t i = 0; i < r; i++)
        for (int64_t j = 0; j < c; j++)
        {
            uint64_t *out = C + (i * c + j) * ccap;
            for (int64_t t = 0; t < ccap; t++)
                out[t] = 0;
            for (int64_t t = lo; t < hi; t++)
            {
                int64_t d0 = t - (len2 - 1);
                if (d0 < 0) d0 = 0;
                int64_t d1 = (t < len1 - 1) ? t : len1 - 1;
                uint64_t acc = 0;
                if (p <= (1ULL << 32))
                {
                    u128 a128 = 0;
                    for (int64_t l = 0; l < k; l++)
                    {
                        const uint64_t *a = A + (i * k + l) * len1;
                        const uint64_t *b = B + (l * c + j) * len2;
                        for (int64_t d = d0; d <= d1; d++)
                            a128 += (u128) (a[d] * b[t - d]);
                    }
                    acc = (uint64_t) (a128 % p);
                }
                else
                {
                    for (int64_t l = 0; l < k; l++)
                    {
                        const uint64_t *a = A + (i * k + l) * len1;
                        const uint64_t *b = B + (l * c + j) * len2;
                        for (int64_t d = d0; d <= d1; d++)
                            acc = addmod(acc, orc_mulmod(a[d], b[t - d], p), p);
                    }
                }
                out[t - lo] = acc;
            }
        }
}

void orc_poly_mat_mul(uint64_t *C, const uint64_t *A, const uint64_t *B,
                      int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                      uint64_t p, int nthreads)
{
    if (len1 <= 0 || len2 <= 0)
        return;
    pm_mul_range(C, len1 + len2 - 1, A, B, r, k, c, len1, len2, 0, len1 + len2 - 1, p, nthreads);
}

int64_t orc_poly_mat_mulmid(uint64_t *res, const uint64_t *A, const uint64_t *B,
                            int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                            int64_t nlo, int64_t nhi, uint64_t p, int nthreads)
{
    const int64_t cap = nhi - nlo;
    if (cap <= 0)
        return 0;
    memset(res, 0, sizeof(uint64_t) * (size_t) (r * c * cap));
    const int64_t L1 = orc_pm_max_length(A, r, k, len1);
    const int64_t L2 = orc_pm_max_length(B, k, c, len2);
    int64_t hi = nhi;
    if (hi > L1 + L2 - 1)
        hi = L1 + L2 - 1;
    if (L1 == 0 || L2 == 0 || nlo >= hi)
        return 0;
    /* compute coefficients [nlo, hi) into a temporary of capacity hi - nlo */
    const int64_t w = hi - nlo;
    uint64_t *tmp = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (r * c * w));
    /* A and B keep their capacities len1/len2 as strides: restrict the
     * convolution to the first L1/L2 coefficients by copying */
    uint64_t *A2 = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (r * k * L1));
    uint64_t *B2 = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (k * c * L2));
    for (int64_t e = 0; e < r * k; e++)
        memcpy(A2 + e * L1, A + e * len1, sizeof(uint64_t) * (size_t) L1);
    for (int64_t e = 0; e < k * c; e++)
        memcpy(B2 + e * L2, B + e * len2, sizeof(uint64_t) * (size_t) L2);
    pm_mul_range(tmp, w, A2, B2, r, k, c, L1, L2, nlo, hi, p, nthreads);
    for (int64_t e = 0; e < r * c; e++)
        memcpy(res + e * cap, tmp + e * w, sizeof(uint64_t) * (size_t) w);
    free(tmp);
    free(A2);
    free(B2);
    return w;
}

/* ------------------------------------------------------------------ */
/* CPU NTT product (port of the evaluation/interpolation pipeline)     */
/* ------------------------------------------------------------------ */

typedef struct
{
    uint32_t p;
    int64_t N;
    int lg;
    uint32_t *w, *wq;      /* forward twiddles per stage, Shoup quotients */
    uint32_t *iw, *iwq;    /* inverse twiddles */
    uint32_t ninv, ninvq;
} cpu_ntt_t;

static inline uint32_t shoup_q(uint32_t w, uint32_t p)
{
    return (uint32_t) (((uint64_t) w << 32) / p);
}

/* x * w mod p in [0, 2p) for x < 2^32 */
static inline uint32_t mul_shoup(uint32_t x, uint32_t w, uint32_t wq, uint32_t p)
{
    uint32_t q = (uint32_t) (((uint64_t) x * wq) >> 32);
    return x * w - q * p;
}

static int cpu_ntt_init(cpu_ntt_t *T, uint32_t p, int64_t N)
{
    int lg = 0;
    while ((1LL << lg) < N) lg++;
    if ((1LL << lg) != N || ((uint64_t) p - 1) % (uint64_t) N != 0)
        return -1;
    /* primitive root: find g whose (p-1)/q powers are != 1 for all prime q | p-1 */
    uint64_t pm1 = p - 1, fac[64];
    int nf = 0;
    {
        uint64_t t = pm1;
        for (uint64_t q = 2; q * q <= t; q++)
            if (t % q == 0) { fac[nf++] = q; while (t % q == 0) t /= q; }
        if (t > 1) fac[nf++] = t;
    }
    uint64_t g = 2;
    for (;; g++)
    {
        int ok = 1;
        for (int i = 0; i < nf; i++)
            if (orc_powmod(g, pm1 / fac[i], p) == 1) { ok = 0; break; }
        if (ok) break;
    }
    uint64_t wN = orc_powmod(g, pm1 / (uint64_t) N, p);
    uint64_t iwN = orc_invmod(wN, p);
    T->p = p; T->N = N; T->lg = lg;
    T->w = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) N);
    T->wq = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) N);
    T->iw = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) N);
    T->iwq = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) N);
    /* table for half size h: entries [h, 2h) hold w_{2h}^j, j < h */
    for (int64_t h = 1; h < N; h <<= 1)
    {
        uint64_t wh = orc_powmod(wN, (uint64_t) (N / (2 * h)), p);
        uint64_t iwh = orc_powmod(iwN, (uint64_t) (N / (2 * h)), p);
        uint64_t x = 1, y = 1;
        for (int64_t j = 0; j < h; j++)
        {
            T->w[h + j] = (uint32_t) x; T->wq[h + j] = shoup_q((uint32_t) x, p);
            T->iw[h + j] = (uint32_t) y; T->iwq[h + j] = shoup_q((uint32_t) y, p);
            x = orc_mulmod(x, wh, p);
            y = orc_mulmod(y, iwh, p);
        }
    }
    T->ninv = (uint32_t) orc_invmod((uint64_t) N % p, p);
    T->ninvq = shoup_q(T->ninv, p);
    return 0;
}

static void cpu_ntt_clear(cpu_ntt_t *T)
{
    free(T->w); free(T->wq); free(T->iw); free(T->iwq);
}

/* forward: natural order in, bit-reversed order out (decimation in frequency) */
static void cpu_ntt_fwd(const cpu_ntt_t *T, uint32_t *a)
{
    const uint32_t p = T->p, p2 = 2 * p;
    for (int64_t h = T->N >> 1; h >= 1; h >>= 1)
        for (int64_t s = 0; s < T->N; s += 2 * h)
            for (int64_t j = 0; j < h; j++)
            {
                uint32_t u = a[s + j], v = a[s + j + h];
                uint32_t x = u + v;
                if (x >= p2) x -= p2;
                uint32_t y = mul_shoup(u + p2 - v, T->w[h + j], T->wq[h + j], p);
                a[s + j] = x;
                a[s + j + h] = y;
            }
    for (int64_t i = 0; i < T->N; i++)
    {
        uint32_t x = a[i];
        if (x >= p) x -= p;
        if (x >= p) x -= p;
        a[i] = x;
    }
}

/* inverse: bit-reversed in, natural out (decimation in time), scaled by 1/N */
static void cpu_ntt_inv(const cpu_ntt_t *T, uint32_t *a)
{
    const uint32_t p = T->p, p2 = 2 * p;
    for (int64_t h = 1; h < T->N; h <<= 1)
        for (int64_t s = 0; s < T->N; s += 2 * h)
            for (int64_t j = 0; j < h; j++)
            {
                uint32_t u = a[s + j];
                if (u >= p2) u -= p2;
                uint32_t v = mul_shoup(a[s + j + h], T->iw[h + j], T->iwq[h + j], p);
                a[s + j] = u + v;
                a[s + j + h] = u + p2 - v;
            }
    for (int64_t i = 0; i < T->N; i++)
    {
        uint32_t x = mul_shoup(a[i], T->ninv, T->ninvq, p);
        if (x >= p) x -= p;
        a[i] = x;
    }
}

/* residues mod q (an NTT prime < 2^30 with N | q - 1) of the coefficients [0, len) of
 * A * B, entry-major with entry stride len; inputs are reduced mod q as they are read */
static int ntt_product_mod_q(uint32_t *out, const uint64_t *A, const uint64_t *B,
                             int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                             uint32_t q, int nthreads)
{
    const int64_t len = len1 + len2 - 1;
    int64_t N = 1;
    while (N < len) N <<= 1;
    cpu_ntt_t T;
    if (cpu_ntt_init(&T, q, N) != 0)
        return -1;
    /* point-major evaluations: E[pt][i][j] */
    uint32_t *EA = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (N * r * k));
    uint32_t *EB = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (N * k * c));
    uint32_t *EC = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (N * r * c));
    const int nt = nthreads > 0 ? nthreads : 1;
    (void) nt;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
        uint32_t *buf = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) N);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t e = 0; e < r * k + k * c; e++)
        {
            const int isA = e < r * k;
            const int64_t ee = isA ? e : e - r * k;
            const uint64_t *src = isA ? A + ee * len1 : B + ee * len2;
            const int64_t L = isA ? len1 : len2;
            for (int64_t d = 0; d < N; d++)
                buf[d] = d < L ? (uint32_t) (src[d] >= q ? src[d] % q : src[d]) : 0;
            cpu_ntt_fwd(&T, buf);
            uint32_t *dst = isA ? EA : EB;
            const int64_t stride = isA ? r * k : k * c;
            for (int64_t d = 0; d < N; d++)
                dst[d * stride + ee] = buf[d];
        }
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t pt = 0; pt < N; pt++)
        {
            const uint32_t *a = EA + pt * r * k, *b = EB + pt * k * c;
            uint32_t *o = EC + pt * r * c;
            for (int64_t i = 0; i < r; i++)
                for (int64_t j = 0; j < c; j++)
                {
                    /* products < 2^60: split every 8 terms, as nmod32_vec/dot_split.c */
                    uint64_t lo = 0, hi = 0;
                    int64_t l = 0;
                    for (; l + 8 <= k; l += 8)
                    {
                        for (int u = 0; u < 8; u++)
                            lo += (uint64_t) a[i * k + l + u] * b[(l + u) * c + j];
                        hi += lo >> 32;
                        lo &= 0xffffffffULL;
                    }
                    for (; l < k; l++)
                        lo += (uint64_t) a[i * k + l] * b[l * c + j];
                    hi += lo >> 32;
                    lo &= 0xffffffffULL;
                    o[i * c + j] = (uint32_t) ((((u128) hi << 32) + lo) % q);
                }
        }
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t e = 0; e < r * c; e++)
        {
            for (int64_t d = 0; d < N; d++)
                buf[d] = EC[d * r * c + e];
            cpu_ntt_inv(&T, buf);
            for (int64_t d = 0; d < len; d++)
                out[e * len + d] = buf[d];
        }
        free(buf);
    }
    free(EA); free(EB); free(EC);
    cpu_ntt_clear(&T);
    return 0;
}

int orc_poly_mat_mul_ntt(uint64_t *C, const uint64_t *A, const uint64_t *B,
                         int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                         uint64_t p, int nthreads)
{
    if (len1 <= 0 || len2 <= 0)
        return 0;
    if (p >= (1ULL << 30))
        return -1;
    const int64_t len = len1 + len2 - 1;
    uint32_t *R = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (r * c * len + 1));
    const int rc = ntt_product_mod_q(R, A, B, r, k, c, len1, len2, (uint32_t) p, nthreads);
    if (rc == 0)
        for (int64_t i = 0; i < r * c * len; i++)
            C[i] = R[i];
    free(R);
    return rc;
}

/* ------------------------------------------------------------------ */
/* multi-prime product for any modulus                                 */
/* ------------------------------------------------------------------ */

/* The NTT primes of the multi-prime product: the largest q = a 2^20 + 1 < 2^30 that are
 * prime, found by a downward search over a (each q > 2^29, transforms up to 2^20). */
#define ORC_CRT_MAXT 6
static uint32_t crt_q[ORC_CRT_MAXT];
static int crt_nq = 0;

static void crt_primes_init(void)
{
    if (crt_nq == ORC_CRT_MAXT)
        return;
    int n = 0;
    uint32_t found[ORC_CRT_MAXT];
    for (uint64_t a = 1023; a >= 512 && n < ORC_CRT_MAXT; a--)
    {
        const uint64_t q = (a << 20) + 1;
        if (orc_is_prime(q))
            found[n++] = (uint32_t) q;
    }
    for (int i = 0; i < n; i++)
        crt_q[i] = found[i];
    crt_nq = n;
}

static int bits_of(uint64_t x)
{
    int b = 0;
    while (x) { b++; x >>= 1; }
    return b;
}

/*
 * C = A * B mod p for any p >= 2: the exact integer product (entries below
 * k * min(len1, len2) * (p-1)^2) modulo t NTT primes, recombined by Garner's mixed
 * radix form and reduced mod p.  This is the multi-prime design of the reference's
 * disabled product (nmod_poly_mat_mul_3_primes.bak:59-153: the prime count from
 * 2 bits(p) + bits(k) + bits(min len)), with primes below 2^30.  Returns -1 when the
 * bound needs more than ORC_CRT_MAXT primes or the transform exceeds 2^20.
 */
int orc_poly_mat_mul_crt(uint64_t *C, const uint64_t *A, const uint64_t *B,
                         int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                         uint64_t p, int nthreads)
{
    if (len1 <= 0 || len2 <= 0)
        return 0;
    const int64_t len = len1 + len2 - 1;
    if (len > (1LL << 20))
        return -1;
    crt_primes_init();
    const int64_t minlen = len1 < len2 ? len1 : len2;
    const int need = bits_of((uint64_t) k) + bits_of((uint64_t) minlen) + 2 * bits_of(p - 1);
    int t = (need + 28) / 29;    /* every prime is > 2^29 */
    if (t < 1) t = 1;
    if (t > crt_nq)
        return -1;
    const int64_t nco = r * c * len;
    uint32_t *R = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (t * nco + 1));
    for (int j = 0; j < t; j++)
        if (ntt_product_mod_q(R + j * nco, A, B, r, k, c, len1, len2, crt_q[j], nthreads) != 0)
        {
            free(R);
            return -1;
        }
    /* inv[j] = (q_0 ... q_{j-1})^-1 mod q_j; qp[j] = q_0 ... q_{j-1} mod p */
    uint64_t inv[ORC_CRT_MAXT], qp[ORC_CRT_MAXT];
    qp[0] = 1 % p;
    inv[0] = 1;
    for (int j = 1; j < t; j++)
    {
        uint64_t pr = 1;
        for (int l = 0; l < j; l++)
            pr = orc_mulmod(pr, crt_q[l] % crt_q[j], crt_q[j]);
        inv[j] = orc_invmod(pr, crt_q[j]);
        qp[j] = orc_mulmod(qp[j - 1], crt_q[j - 1] % p, p);
    }
    const int nt = nthreads > 0 ? nthreads : 1;
    (void) nt;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nt)
#endif
    for (int64_t i = 0; i < nco; i++)
    {
        uint64_t v[ORC_CRT_MAXT];
        v[0] = R[i];
        for (int j = 1; j < t; j++)
        {
            const uint64_t qj = crt_q[j];
            /* (v_0 + v_1 q_0 + ... + v_{j-1} q_0..q_{j-2}) mod q_j by Horner */
            uint64_t acc = v[j - 1] % qj;
            for (int l = j - 2; l >= 0; l--)
                acc = (orc_mulmod(acc, crt_q[l], qj) + v[l]) % qj;
            const uint64_t rj = R[j * nco + i];
            v[j] = orc_mulmod((rj + qj - acc) % qj, inv[j], qj);
        }
        /* x = sum_j v_j (q_0 .. q_{j-1}) mod p */
        uint64_t x = 0;
        for (int j = 0; j < t; j++)
            x = addmod(x, orc_mulmod(v[j] % p, qp[j], p), p);
        C[i] = x;
    }
    free(R);
    return 0;
}

/* product used inside pmbasis: NTT port when applicable, else schoolbook */
static void pm_mul_auto(uint64_t *C, const uint64_t *A, const uint64_t *B,
                        int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                        uint64_t p, int nthreads)
{
    if (len1 <= 0 || len2 <= 0)
        return;
    if ((int64_t) r * k * c * len1 * len2 > (1LL << 22)
        && (orc_poly_mat_mul_ntt(C, A, B, r, k, c, len1, len2, p, nthreads) == 0
            || orc_poly_mat_mul_crt(C, A, B, r, k, c, len1, len2, p, nthreads) == 0))
        return;
    orc_poly_mat_mul(C, A, B, r, k, c, len1, len2, p, nthreads);
}

/* ------------------------------------------------------------------ */
/* mbasis / pmbasis                                                    */
/* ------------------------------------------------------------------ */

/* stable permutation sorting (shift[i], i) increasingly;
 * _find_shift_permutation, nmod_mat_poly_mbasis.c:69-114 */
static void shift_permutation(int64_t *perm, const int64_t *shift, int64_t m)
{
    for (int64_t i = 0; i < m; i++)
        perm[i] = i;
    for (int64_t i = 1; i < m; i++)
    {
        int64_t x = perm[i], j = i - 1;
        while (j >= 0 && (shift[perm[j]] > shift[x]
                          || (shift[perm[j]] == shift[x] && perm[j] > x)))
        {
            perm[j + 1] = perm[j];
            j--;
        }
        perm[j + 1] = x;
    }
}

/*
 * Iterative order-1 steps.  appbas is kept coefficient-major (ab[d][i][j], the
 * nmod_mat_poly_t layout of nmod_mat_poly.h:70-78) with capacity order+1.
 * F is entry-major (input layout), capacity flen.
 */
int64_t orc_mbasis(uint64_t *appbas, int64_t *shift, const uint64_t *F,
                   int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p)
{
    const int64_t cap = order + 1;
    memset(appbas, 0, sizeof(uint64_t) * (size_t) (m * m * cap));
    for (int64_t i = 0; i < m; i++)
        appbas[(i * m + i) * cap] = 1 % p;
    if (order <= 0)
        return (p == 1) ? 0 : 1;

    /* matp = set_trunc_from_poly_mat(F, order), coefficient-major */
    const int64_t fl = flen < order ? flen : order;
    uint64_t *Fc = (uint64_t *) calloc((size_t) (fl * m * n + 1), sizeof(uint64_t));
    int is_zero = 1;
    for (int64_t i = 0; i < m; i++)
        for (int64_t j = 0; j < n; j++)
            for (int64_t d = 0; d < fl; d++)
            {
                uint64_t v = F[(i * n + j) * flen + d];
                Fc[d * m * n + i * n + j] = v;
                if (v) is_zero = 0;
            }
    if (is_zero)
    {
        free(Fc);
        return 1;
    }

    uint64_t *ab = (uint64_t *) calloc((size_t) (cap * m * m), sizeof(uint64_t));
    for (int64_t i = 0; i < m; i++)
        ab[i * m + i] = 1;
    int64_t alen = 1;

    uint64_t *res = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * n));
    uint64_t *tmp = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * (n > m ? n : m)));
    uint64_t *nsbas = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m + 1));
    uint64_t *rowbuf = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m));
    int64_t *perm = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    int64_t *piv = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    int64_t *ipiv = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);

    for (int64_t ord = 0; ord < order; ord++)
    {
        /* residual: coefficient ord of appbas * matp (nmod_mat_poly_arith.c:4-41) */
        memset(res, 0, sizeof(uint64_t) * (size_t) (m * n));
        {
            int64_t ub = (ord + 1 < alen) ? ord + 1 : alen;
            int64_t lb = ord + 1 - fl;
            if (lb < 0) lb = 0;
            for (int64_t t = lb; t < ub; t++)
            {
                orc_nmod_mat_mul(tmp, ab + t * m * m, Fc + (ord - t) * m * n, m, m, n, p);
                for (int64_t e = 0; e < m * n; e++)
                    res[e] = addmod(res[e], tmp[e], p);
            }
        }
        /* permute rows of res by the stable shift sort */
        shift_permutation(perm, shift, m);
        for (int64_t i = 0; i < m; i++)
            memcpy(tmp + i * n, res + perm[i] * n, sizeof(uint64_t) * (size_t) n);
        memcpy(res, tmp, sizeof(uint64_t) * (size_t) (m * n));

        const int64_t nullity = orc_left_nullspace_compact(nsbas, piv, res, m, n, p);
        const int64_t rank = m - nullity;

        if (nullity == 0)
        {
            /* appbas = X^(order-ord) * appbas; shift += order-ord (:221-231) */
            const int64_t sh = order - ord;
            for (int64_t d = alen - 1; d >= 0; d--)
                memcpy(ab + (d + sh) * m * m, ab + d * m * m, sizeof(uint64_t) * (size_t) (m * m));
            memset(ab, 0, sizeof(uint64_t) * (size_t) (sh * m * m));
            alen += sh;
            for (int64_t i = 0; i < m; i++)
                shift[i] += sh;
            break;
        }
        else if (nullity < m)
        {
            /* pivots <- perm o pivots; shift[pivots[i]]++ for i < rank (:252-267) */
            for (int64_t i = 0; i < m; i++)
                piv[i] = perm[piv[i]];
            for (int64_t i = 0; i < rank; i++)
                shift[piv[i]] += 1;
            /* permute rows of appbas: new row i = old row piv[i] */
            for (int64_t d = 0; d < alen; d++)
            {
                uint64_t *M = ab + d * m * m;
                for (int64_t i = 0; i < m; i++)
                    memcpy(rowbuf + i * m, M + piv[i] * m, sizeof(uint64_t) * (size_t) m);
                memcpy(M, rowbuf, sizeof(uint64_t) * (size_t) (m * m));
            }
            /* rows[rank..m) += nsbas * rows[0..rank), per coefficient (:296-304) */
            for (int64_t d = 0; d < alen; d++)
            {
                uint64_t *M = ab + d * m * m;
                orc_nmod_mat_mul(rowbuf, nsbas, M, nullity, rank, m, p);
                for (int64_t e = 0; e < nullity * m; e++)
                    M[rank * m + e] = addmod(M[rank * m + e], rowbuf[e], p);
            }
            /* grow the length if one of rows[0..rank) reaches the top coefficient */
            {
                const uint64_t *top = ab + (alen - 1) * m * m;
                int grow = 0;
                for (int64_t e = 0; e < rank * m && !grow; e++)
                    if (top[e]) grow = 1;
                if (grow)
                {
                    memset(ab + alen * m * m, 0, sizeof(uint64_t) * (size_t) (m * m));
                    alen++;
                }
            }
            /* rows[0..rank) *= X */
            for (int64_t d = alen - 1; d > 0; d--)
                memcpy(ab + d * m * m, ab + (d - 1) * m * m, sizeof(uint64_t) * (size_t) (rank * m));
            memset(ab, 0, sizeof(uint64_t) * (size_t) (rank * m));
            /* un-permute: rows back to their original positions */
            for (int64_t i = 0; i < m; i++)
                ipiv[piv[i]] = i;
            for (int64_t d = 0; d < alen; d++)
            {
                uint64_t *M = ab + d * m * m;
                for (int64_t i = 0; i < m; i++)
                    memcpy(rowbuf + i * m, M + ipiv[i] * m, sizeof(uint64_t) * (size_t) m);
                memcpy(M, rowbuf, sizeof(uint64_t) * (size_t) (m * m));
            }
        }
    }

    /* nmod_poly_mat_set_from_mat_poly: back to entry-major */
    for (int64_t i = 0; i < m; i++)
        for (int64_t j = 0; j < m; j++)
            for (int64_t d = 0; d < alen && d < cap; d++)
                appbas[(i * m + j) * cap + d] = ab[d * m * m + i * m + j];

    free(Fc); free(ab); free(res); free(tmp); free(nsbas); free(rowbuf);
    free(perm); free(piv); free(ipiv);
    return orc_pm_max_length(appbas, m, m, cap);
}

/* copy entry-major P (capacity pc) into a fresh buffer of capacity nc */
static uint64_t *pm_recap(const uint64_t *P, int64_t r, int64_t c, int64_t pc, int64_t nc)
{
    uint64_t *Q = (uint64_t *) calloc((size_t) (r * c * nc + 1), sizeof(uint64_t));
    const int64_t l = pc < nc ? pc : nc;
    for (int64_t e = 0; e < r * c; e++)
        memcpy(Q + e * nc, P + e * pc, sizeof(uint64_t) * (size_t) l);
    return Q;
}

int64_t orc_pmbasis(uint64_t *appbas, int64_t *shift, const uint64_t *F,
                    int64_t m, int64_t n, int64_t flen, int64_t order, uint64_t p,
                    int64_t thres, int nthreads)
{
    const int64_t cap = order + 1;
    if (thres < 1)
        thres = 1;
    /* pmat = set_trunc(F, order) */
    const int64_t pl = flen < order ? flen : order;
    if (order <= thres)
        return orc_mbasis(appbas, shift, F, m, n, flen, order, p);

    const int64_t order1 = order >> 1;
    const int64_t order2 = order - order1;
    uint64_t *pmat = pm_recap(F, m, n, flen, pl > 0 ? pl : 1);
    const int64_t plc = pl > 0 ? pl : 1;

    uint64_t *A1 = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m * (order1 + 1)));
    int64_t l1 = orc_pmbasis(A1, shift, pmat, m, n, plc, order1, p, thres, nthreads);
    if (l1 < 1) l1 = 1;
    uint64_t *A1t = pm_recap(A1, m, m, order1 + 1, l1);

    /* residual = mulmid(appbas, pmat, order1, order) */
    uint64_t *res = (uint64_t *) calloc((size_t) (m * n * order2), sizeof(uint64_t));
    {
        const int64_t L2 = orc_pm_max_length(pmat, m, n, plc);
        int64_t hi = order;
        if (hi > l1 + L2 - 1) hi = l1 + L2 - 1;
        if (L2 > 0 && hi > order1)
        {
            uint64_t *full = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * n * (l1 + L2 - 1)));
            uint64_t *Bt = pm_recap(pmat, m, n, plc, L2);
            pm_mul_auto(full, A1t, Bt, m, m, n, l1, L2, p, nthreads);
            for (int64_t e = 0; e < m * n; e++)
                for (int64_t t = order1; t < hi; t++)
                    res[e * order2 + t - order1] = full[e * (l1 + L2 - 1) + t];
            free(full);
            free(Bt);
        }
    }

    uint64_t *A2 = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m * (order2 + 1)));
    int64_t l2 = orc_pmbasis(A2, shift, res, m, n, order2, order2, p, thres, nthreads);
    if (l2 < 1) l2 = 1;
    uint64_t *A2t = pm_recap(A2, m, m, order2 + 1, l2);

    /* appbas = appbas2 * appbas */
    const int64_t lp = l1 + l2 - 1;
    uint64_t *prod = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m * lp));
    pm_mul_auto(prod, A2t, A1t, m, m, m, l2, l1, p, nthreads);
    memset(appbas, 0, sizeof(uint64_t) * (size_t) (m * m * cap));
    for (int64_t e = 0; e < m * m; e++)
        for (int64_t d = 0; d < lp && d < cap; d++)
            appbas[e * cap + d] = prod[e * lp + d];

    free(pmat); free(A1); free(A1t); free(res); free(A2); free(A2t); free(prod);
    return orc_pm_max_length(appbas, m, m, cap);
}

/* ------------------------------------------------------------------ */
/* approximant basis verifier (verification.c:21-116)                  */
/* ------------------------------------------------------------------ */

static int64_t poly_deg(const uint64_t *a, int64_t cap)
{
    int64_t d = cap - 1;
    while (d >= 0 && a[d] == 0)
        d--;
    return d;
}

/* determinant of an m x m matrix mod p (prime) by elimination */
static uint64_t det_mod(uint64_t *M, int64_t m, uint64_t p)
{
    uint64_t det = 1 % p;
    for (int64_t col = 0; col < m; col++)
    {
        int64_t piv = -1;
        for (int64_t i = col; i < m; i++)
            if (M[i * m + col]) { piv = i; break; }
        if (piv < 0)
            return 0;
        if (piv != col)
        {
            for (int64_t j = 0; j < m; j++)
            {
                uint64_t t = M[piv * m + j];
                M[piv * m + j] = M[col * m + j];
                M[col * m + j] = t;
            }
            det = det ? p - det : 0;
        }
        det = orc_mulmod(det, M[col * m + col], p);
        uint64_t inv = orc_invmod(M[col * m + col], p);
        for (int64_t i = col + 1; i < m; i++)
        {
            uint64_t f = orc_mulmod(M[i * m + col], inv, p);
            if (!f) continue;
            for (int64_t j = col; j < m; j++)
                M[i * m + j] = submod(M[i * m + j], orc_mulmod(f, M[col * m + j], p), p);
        }
    }
    return det;
}

int orc_is_approximant_basis(const uint64_t *appbas, int64_t alen,
                             const uint64_t *F, int64_t flen,
                             int64_t m, int64_t n, int64_t order,
                             const int64_t *shift_in, uint64_t p)
{
    int fail = 0;
    if (alen < 1)
        return 1 | 4 | 8;

    /* ordered weak Popov, ROW_LOWER: shifted pivot index = largest column
     * reaching the shifted row degree; pivot indices strictly increasing, no
     * zero row (nmod_poly_mat_is_form.c:89-117) */
    {
        int64_t prev = -1;
        for (int64_t i = 0; i < m; i++)
        {
            int64_t best = INT64_MIN, pj = -1;
            for (int64_t j = 0; j < m; j++)
            {
                int64_t d = poly_deg(appbas + (i * m + j) * alen, alen);
                if (d < 0) continue;
                if (d + shift_in[j] >= best) { best = d + shift_in[j]; pj = j; }
            }
            if (pj < 0 || pj <= prev) { fail |= 1; break; }
            prev = pj;
        }
    }

    /* residual = appbas * F; coefficients below order must vanish */
    const int64_t rl = alen + flen - 1;
    uint64_t *resid = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * n * rl));
    pm_mul_auto(resid, appbas, F, m, m, n, alen, flen, p, 1);
    for (int64_t e = 0; e < m * n && !(fail & 2); e++)
        for (int64_t t = 0; t < order && t < rl; t++)
            if (resid[e * rl + t]) { fail |= 2; break; }

    /* det(appbas) has degree sum of diagonal degrees: evaluate at B+1 points */
    {
        int64_t D = 0, B = 0;
        for (int64_t i = 0; i < m; i++)
        {
            D += poly_deg(appbas + (i * m + i) * alen, alen);
            int64_t rd = -1;
            for (int64_t j = 0; j < m; j++)
            {
                int64_t d = poly_deg(appbas + (i * m + j) * alen, alen);
                if (d > rd) rd = d;
            }
            B += rd > 0 ? rd : 0;
        }
        if ((uint64_t) B + 1 < p && B < 4096)
        {
            /* det(x) sampled at x = 1..B+1, interpolated by Newton's divided
             * differences, degree read off the coefficients */
            const int64_t np = B + 1;
            uint64_t *vals = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) np);
            uint64_t *M = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m));
            for (int64_t t = 0; t < np; t++)
            {
                const uint64_t x = (uint64_t) (t + 1);
                for (int64_t e = 0; e < m * m; e++)
                {
                    uint64_t acc = 0;
                    for (int64_t d = alen - 1; d >= 0; d--)
                        acc = addmod(orc_mulmod(acc, x, p), appbas[e * alen + d], p);
                    M[e] = acc;
                }
                vals[t] = det_mod(M, m, p);
            }
            /* Newton divided differences in place */
            for (int64_t j = 1; j < np; j++)
                for (int64_t t = np - 1; t >= j; t--)
                {
                    uint64_t num = submod(vals[t], vals[t - 1], p);
                    uint64_t den = (uint64_t) j % p; /* x_t - x_{t-j} = j */
                    vals[t] = orc_mulmod(num, orc_invmod(den, p), p);
                }
            /* Newton form -> monomial coefficients */
            uint64_t *coef = (uint64_t *) calloc((size_t) np, sizeof(uint64_t));
            for (int64_t j = np - 1; j >= 0; j--)
            {
                /* coef = coef * (x - x_j) + vals[j], x_j = j+1 */
                const uint64_t xj = (uint64_t) (j + 1) % p;
                for (int64_t d = np - 1; d >= 1; d--)
                    coef[d] = submod(coef[d - 1], orc_mulmod(coef[d], xj, p), p);
                coef[0] = submod(vals[j], orc_mulmod(coef[0], xj, p), p);
            }
            if (poly_deg(coef, np) != D)
                fail |= 4;
            free(coef); free(vals); free(M);
        }
    }

    /* [appbas(0) | coeff_order(appbas * F)] has full rank m */
    {
        uint64_t *CP = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * (m + n)));
        for (int64_t i = 0; i < m; i++)
        {
            for (int64_t j = 0; j < m; j++)
                CP[i * (m + n) + j] = appbas[(i * m + j) * alen];
            for (int64_t j = 0; j < n; j++)
                CP[i * (m + n) + m + j] = (order < rl) ? resid[(i * n + j) * rl + order] : 0;
        }
        if (orc_nmod_mat_rank(CP, m, m + n, p) != m)
            fail |= 8;
        free(CP);
    }
    free(resid);
    return fail;
}

/* ------------------------------------------------------------------ */
/* dot products                                                        */
/* ------------------------------------------------------------------ */

uint64_t orc_nmod_vec_dot(const uint64_t *v1, const uint64_t *v2, int64_t len, uint64_t p)
{
    /* exact 192-bit accumulation, one reduction at the end */
    uint64_t r[3];
    orc_integer_dot(r, v1, v2, len);
    /* (r2*2^128 + r1*2^64 + r0) mod p by Horner on 64-bit limbs */
    u128 acc = r[2] % p;
    acc = ((acc << 64) | r[1]) % p;
    acc = ((acc << 64) | r[0]) % p;
    return (uint64_t) acc;
}

/* uv[j] = sum_{i<len} u[i] v[i*k + j] mod p, j < k (nmod_vec_dot_product_multi,
 * nmod_vec_dot_product_multi.c:2054, with the rows of v contiguous): every column an
 * exact 192-bit sum reduced once, columns in parallel */
void orc_nmod_vec_dot_multi(uint64_t *uv, const uint64_t *u, const uint64_t *v, int64_t len, int64_t k,
                            uint64_t p, int nthreads)
{
    (void) nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int64_t j = 0; j < k; j++)
    {
        uint64_t r0 = 0, r1 = 0, r2 = 0;
        for (int64_t i = 0; i < len; i++)
        {
            const u128 t = (u128) u[i] * v[i * k + j];
            const uint64_t lo = (uint64_t) t, hi = (uint64_t) (t >> 64);
            r0 += lo;
            const uint64_t h = hi + (r0 < lo);   /* hi <= 2^64 - 2: no wrap */
            r1 += h;
            r2 += r1 < h;
        }
        u128 acc = r2 % p;
        acc = ((acc << 64) | r1) % p;
        acc = ((acc << 64) | r0) % p;
        uv[j] = (uint64_t) acc;
    }
}

uint32_t orc_nmod32_vec_dot(const uint32_t *v1, const uint32_t *v2, int64_t len, uint64_t p)
{
    u128 acc = 0;
    for (int64_t i = 0; i < len; i++)
        acc += (uint64_t) v1[i] * v2[i];
    return (uint32_t) (acc % p);
}

void orc_integer_dot(uint64_t res[3], const uint64_t *v1, const uint64_t *v2, int64_t len)
{
    uint64_t r0 = 0, r1 = 0, r2 = 0;
    for (int64_t i = 0; i < len; i++)
    {
        u128 pr = (u128) v1[i] * v2[i];
        u128 s = (u128) r0 + (uint64_t) pr;
        r0 = (uint64_t) s;
        u128 s1 = (u128) r1 + (uint64_t) (pr >> 64) + (uint64_t) (s >> 64);
        r1 = (uint64_t) s1;
        r2 += (uint64_t) (s1 >> 64);
    }
    res[0] = r0; res[1] = r1; res[2] = r2;
}

void orc_nmod32_vec_mdot(uint32_t *mv, const uint32_t *mat, const uint32_t *vec,
                         int64_t nrows, int64_t len, int64_t stride, uint64_t p)
{
    for (int64_t i = 0; i < nrows; i++)
        mv[i] = orc_nmod32_vec_dot(mat + i * stride, vec, len, p);
}

/* ------------------------------------------------------------------ */
/* multimodular reduction and CRT                                      */
/* ------------------------------------------------------------------ */

void orc_multimod_reduce(uint64_t *residues, const uint64_t *input, int64_t nb,
                         const uint64_t *primes, int nprimes)
{
    for (int j = 0; j < nprimes; j++)
        for (int64_t i = 0; i < nb; i++)
            residues[j * nb + i] = input[i] % primes[j];
}

void orc_multimod_crt(uint64_t *out, const uint64_t *residues, int64_t nb,
                      const uint64_t *primes, int nprimes, uint64_t p)
{
    /* Garner: x = c0 + c1 q0 + c2 q0 q1 + ..., then Horner mod p */
    uint64_t cinv[16];
    for (int j = 1; j < nprimes; j++)
    {
        uint64_t pr = 1;
        for (int l = 0; l < j; l++)
            pr = orc_mulmod(pr, primes[l] % primes[j], primes[j]);
        cinv[j] = orc_invmod(pr, primes[j]);
    }
    for (int64_t i = 0; i < nb; i++)
    {
        uint64_t cdig[16];
        for (int j = 0; j < nprimes; j++)
        {
            const uint64_t q = primes[j];
            /* value of the partial mixed-radix number mod q */
            uint64_t v = 0;
            for (int l = j - 1; l >= 0; l--)
                v = addmod(orc_mulmod(v, primes[l] % q, q), cdig[l] % q, q);
            uint64_t r = residues[j * nb + i] % q;
            cdig[j] = (j == 0) ? r : orc_mulmod(submod(r, v, q), cinv[j], q);
        }
        uint64_t x = 0;
        for (int l = nprimes - 1; l >= 0; l--)
            x = addmod(orc_mulmod(x, primes[l] % p, p), cdig[l] % p, p);
        out[i] = x;
    }
}

/* ------------------------------------------------------------------ */
/* kernel basis, Zhou-Labahn-Storjohann via approximant bases          */
/* (nmod_poly_mat_kernel_zls_approx, kernel.c:232-480)                 */
/* ------------------------------------------------------------------ */

/* a polynomial matrix: entry (i, j) at a + (i * c + j) * cap */
typedef struct
{
    uint64_t *a;
    int64_t r, c, cap;
} kpm_t;

static kpm_t kpm_zero(int64_t r, int64_t c, int64_t cap)
{
    kpm_t P;
    P.r = r; P.c = c; P.cap = cap > 0 ? cap : 1;
    P.a = (uint64_t *) calloc((size_t) (r * c * P.cap + 1), sizeof(uint64_t));
    return P;
}

static void kpm_free(kpm_t *P)
{
    free(P->a);
    P->a = NULL;
}

static kpm_t kpm_identity(int64_t m)
{
    kpm_t P = kpm_zero(m, m, 1);
    for (int64_t i = 0; i < m; i++)
        P.a[(i * m + i) * P.cap] = 1;
    return P;
}

static int64_t kpm_len(const kpm_t *P)
{
    return orc_pm_max_length(P->a, P->r, P->c, P->cap);
}

/* rows [r0, r1) and columns [c0, c1), capacity kept */
static kpm_t kpm_window(const kpm_t *P, int64_t r0, int64_t r1, int64_t c0, int64_t c1)
{
    kpm_t Q = kpm_zero(r1 - r0, c1 - c0, P->cap);
    for (int64_t i = r0; i < r1; i++)
        for (int64_t j = c0; j < c1; j++)
            memcpy(Q.a + ((i - r0) * Q.c + (j - c0)) * Q.cap, P->a + (i * P->c + j) * P->cap,
                   sizeof(uint64_t) * (size_t) P->cap);
    return Q;
}

/* A * B (nmod_poly_mat_multiply) */
static kpm_t kpm_mul(const kpm_t *A, const kpm_t *B, uint64_t p, int nthreads)
{
    const int64_t la = kpm_len(A), lb = kpm_len(B);
    if (la == 0 || lb == 0)
        return kpm_zero(A->r, B->c, 1);
    uint64_t *At = pm_recap(A->a, A->r, A->c, A->cap, la);
    uint64_t *Bt = pm_recap(B->a, B->r, B->c, B->cap, lb);
    kpm_t C = kpm_zero(A->r, B->c, la + lb - 1);
    pm_mul_auto(C.a, At, Bt, A->r, A->c, B->c, la, lb, p, nthreads);
    free(At); free(Bt);
    return C;
}

/* rows[i] <- rows[perm[i]] for i < nrows, and store[i] <- store[perm[i]]
 * (nmod_poly_mat_permute_rows, nmod_poly_mat_utils.h:264) */
static void kpm_permute_rows(kpm_t *P, int64_t nrows, const int64_t *perm, int64_t *store)
{
    const size_t row = (size_t) (P->c * P->cap);
    uint64_t *tmp = (uint64_t *) malloc(sizeof(uint64_t) * row * (size_t) (nrows > 0 ? nrows : 1));
    for (int64_t i = 0; i < nrows; i++)
        memcpy(tmp + (size_t) i * row, P->a + (size_t) perm[i] * row, sizeof(uint64_t) * row);
    memcpy(P->a, tmp, sizeof(uint64_t) * row * (size_t) nrows);
    free(tmp);
    if (store)
    {
        int64_t *t = (int64_t *) malloc(sizeof(int64_t) * (size_t) (nrows > 0 ? nrows : 1));
        for (int64_t i = 0; i < nrows; i++)
            t[i] = store[perm[i]];
        memcpy(store, t, sizeof(int64_t) * (size_t) nrows);
        free(t);
    }
}

/* rows [0, k) of P replaced by the rows of Q (same column count), capacity grown as needed */
static void kpm_set_rows(kpm_t *P, const kpm_t *Q, int64_t k)
{
    if (Q->cap > P->cap)
    {
        uint64_t *a = pm_recap(P->a, P->r, P->c, P->cap, Q->cap);
        free(P->a);
        P->a = a;
        P->cap = Q->cap;
    }
    for (int64_t i = 0; i < k; i++)
        for (int64_t j = 0; j < P->c; j++)
        {
            uint64_t *d = P->a + (i * P->c + j) * P->cap;
            memset(d, 0, sizeof(uint64_t) * (size_t) P->cap);
            memcpy(d, Q->a + (i * Q->c + j) * Q->cap, sizeof(uint64_t) * (size_t) Q->cap);
        }
}

static int64_t kzls(kpm_t *ker, int64_t *pivind, int64_t *shift, const kpm_t *pm, uint64_t p, int nt)
{
    const int64_t m = pm->r, n = pm->c;
    /* empty matrices, or single row/column vectors that are zero (:240-248) */
    if (m == 0 || n == 0 || ((m == 1 || n == 1) && kpm_len(pm) == 0))
    {
        *ker = kpm_identity(m);
        for (int64_t i = 0; i < m; i++)
            pivind[i] = i;
        return m;
    }
    /* one nonzero row (:251-252) */
    if (m == 1)
    {
        *ker = kpm_zero(m, m, 1);
        return 0;
    }
    /* 2n > m: split the columns [n - n/2 | n/2] (:256-317) */
    if (2 * n > m)
    {
        const int64_t n1 = n - n / 2;
        kpm_t left = kpm_window(pm, 0, m, 0, n1);
        kpm_t k1;
        int64_t nullity = kzls(&k1, pivind, shift, &left, p, nt);
        kpm_free(&left);
        if (nullity == 0)
        {
            *ker = k1;
            return 0;
        }
        kpm_t ker1 = kpm_window(&k1, 0, nullity, 0, m);
        kpm_t right = kpm_window(pm, 0, m, n1, n);
        kpm_t resid = kpm_mul(&ker1, &right, p, nt);
        kpm_free(&right);
        kpm_t k2;
        int64_t *piv2 = (int64_t *) malloc(sizeof(int64_t) * (size_t) nullity);
        const int64_t nullity2 = kzls(&k2, piv2, shift, &resid, p, nt);
        kpm_free(&resid);
        if (nullity2 > 0)
        {
            kpm_t k2top = kpm_window(&k2, 0, nullity2, 0, nullity);
            kpm_t k3 = kpm_mul(&k2top, &ker1, p, nt);
            kpm_set_rows(&k1, &k3, nullity2);
            for (int64_t i = 0; i < nullity2; i++)
                pivind[i] = pivind[piv2[i]];
            kpm_free(&k2top);
            kpm_free(&k3);
        }
        kpm_free(&k2);
        kpm_free(&ker1);
        free(piv2);
        *ker = k1;
        return nullity2;
    }

    /* 1 <= n <= m/2 (:321-479) */
    int64_t *buf = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    int64_t nnz = 0;
    for (int64_t i = 0; i < m; i++)
    {
        int64_t mx = -1;
        for (int64_t j = 0; j < n; j++)
        {
            const int64_t d = poly_deg(pm->a + (i * n + j) * pm->cap, pm->cap);
            if (d > mx) mx = d;
        }
        if (mx >= 0) { nnz++; buf[i] = mx; }
        else buf[i] = 0;
    }
    if (nnz == 0)
    {
        *ker = kpm_identity(m);
        for (int64_t i = 0; i < m; i++)
            pivind[i] = i;
        free(buf);
        return m;
    }
    int64_t maxdeg = buf[0], diff_shift = shift[0] - buf[0];
    for (int64_t i = 1; i < m; i++)
    {
        if (buf[i] > maxdeg) maxdeg = buf[i];
        if (diff_shift > shift[i] - buf[i]) diff_shift = shift[i] - buf[i];
    }
    /* order = 1 + max(maxdeg, 1 + floor((sum(shift) - m * diff_shift - 1) / (m - n)))
     * with C's truncating division, as the reference computes it (:352-356) */
    int64_t order = -m * diff_shift - 1;
    for (int64_t i = 0; i < m; i++)
        order += shift[i];
    order = 1 + order / (m - n);
    order = 1 + (maxdeg > order ? maxdeg : order);

    const int64_t plen = kpm_len(pm) > 0 ? kpm_len(pm) : 1;
    uint64_t *pmt = pm_recap(pm->a, m, n, pm->cap, plen);
    kpm_t K = kpm_zero(m, m, order + 1);
    orc_pmbasis(K.a, shift, pmt, m, n, plen, order, p, 32, nt);

    /* rows of the approximant basis that are kernel rows (:361-382) */
    int64_t nullity = 0, sum_pmatdeg = 0;
    int no_constant_pivot_and_row = 1;
    for (int64_t i = 0; i < m; i++)
    {
        if (shift[i] < order + diff_shift)
            pivind[nullity++] = i;
        else
        {
            if (buf[i] == 0 && poly_deg(K.a + (i * m + i) * K.cap, K.cap) <= 0)
                no_constant_pivot_and_row = 0;
            sum_pmatdeg += buf[i];
            buf[i - nullity] = i;
        }
    }
    for (int64_t i = nullity; i < m; i++)
        pivind[i] = buf[i - nullity];
    kpm_permute_rows(&K, m, pivind, shift);

    /* early exit (:392-404) */
    if (nullity >= m - n && no_constant_pivot_and_row)
    {
        int64_t sum_pivdeg = 0;
        for (int64_t i = 0; i < nullity; i++)
            sum_pivdeg += poly_deg(K.a + (i * m + pivind[i]) * K.cap, K.cap);
        if (sum_pivdeg == sum_pmatdeg)
        {
            free(buf); free(pmt);
            *ker = K;
            return nullity;
        }
    }

    /* residual of the other rows, its kernel, and the missing kernel rows (:406-441) */
    kpm_t approx = kpm_window(&K, nullity, m, 0, m);
    kpm_t resid = kpm_zero(m - nullity, n, maxdeg + 1);
    {
        const int64_t la = kpm_len(&approx) > 0 ? kpm_len(&approx) : 1;
        uint64_t *At = pm_recap(approx.a, m - nullity, m, approx.cap, la);
        orc_poly_mat_mulmid(resid.a, At, pmt, m - nullity, m, n, la, plen, order, order + maxdeg + 1, p, nt);
        free(At);
    }
    kpm_t k2;
    const int64_t nullity2 = kzls(&k2, buf, shift + nullity, &resid, p, nt);
    kpm_free(&resid);
    if (nullity2 == 0)
    {
        kpm_free(&k2); kpm_free(&approx); free(buf); free(pmt);
        *ker = K;
        return nullity;
    }
    {
        kpm_t k2top = kpm_window(&k2, 0, nullity2, 0, m - nullity);
        kpm_t prod = kpm_mul(&k2top, &approx, p, nt);
        /* rows [nullity, nullity + nullity2) of K <- prod */
        kpm_t tail = kpm_window(&K, nullity, m, 0, m);
        kpm_set_rows(&tail, &prod, nullity2);
        if (tail.cap > K.cap)
        {
            uint64_t *a = pm_recap(K.a, m, m, K.cap, tail.cap);
            free(K.a);
            K.a = a;
            K.cap = tail.cap;
        }
        for (int64_t i = 0; i < m - nullity; i++)
            for (int64_t j = 0; j < m; j++)
            {
                uint64_t *d = K.a + ((nullity + i) * m + j) * K.cap;
                memset(d, 0, sizeof(uint64_t) * (size_t) K.cap);
                memcpy(d, tail.a + (i * m + j) * tail.cap, sizeof(uint64_t) * (size_t) tail.cap);
            }
        kpm_free(&k2top); kpm_free(&prod); kpm_free(&tail);
    }
    for (int64_t i = 0; i < nullity2; i++)
        pivind[nullity + i] = pivind[nullity + buf[i]];

    /* merge the two sorted pivot lists, permuting rows, pivots and shifts (:443-468) */
    const int64_t tot = nullity + nullity2;
    int64_t i1 = 0, i2 = 0;
    for (int64_t i = 0; i < tot; i++)
    {
        if (i2 == nullity2 || (i1 < nullity && pivind[i1] < pivind[nullity + i2]))
            buf[i] = i1++;
        else
            buf[i] = nullity + i2++;
    }
    kpm_permute_rows(&K, tot, buf, NULL);
    int64_t *t = (int64_t *) malloc(sizeof(int64_t) * (size_t) tot);
    for (int64_t i = 0; i < tot; i++) t[i] = pivind[i];
    for (int64_t i = 0; i < tot; i++) pivind[i] = t[buf[i]];
    for (int64_t i = 0; i < tot; i++) t[i] = shift[i];
    for (int64_t i = 0; i < tot; i++) shift[i] = t[buf[i]];
    free(t);
    kpm_free(&k2); kpm_free(&approx); free(buf); free(pmt);
    *ker = K;
    return tot;
}

int64_t orc_kernel_zls(uint64_t **ker, int64_t *klen, int64_t *pivind, int64_t *shift,
                       const uint64_t *pmat, int64_t m, int64_t n, int64_t plen, uint64_t p,
                       int nthreads)
{
    kpm_t P;
    P.r = m; P.c = n; P.cap = plen > 0 ? plen : 1;
    P.a = pm_recap(pmat, m, n, plen > 0 ? plen : 0, P.cap);
    kpm_t K;
    const int64_t nullity = kzls(&K, pivind, shift, &P, p, nthreads);
    kpm_free(&P);
    /* the kernel rows, capacity their max length (at least 1); other rows zero */
    kpm_t rows = kpm_window(&K, 0, nullity, 0, m);
    const int64_t L = kpm_len(&rows) > 0 ? kpm_len(&rows) : 1;
    uint64_t *out = (uint64_t *) calloc((size_t) (m * m * L + 1), sizeof(uint64_t));
    for (int64_t e = 0; e < nullity * m; e++)
        memcpy(out + e * L, rows.a + e * rows.cap, sizeof(uint64_t) * (size_t) (L < rows.cap ? L : rows.cap));
    kpm_free(&rows);
    kpm_free(&K);
    *ker = out;
    *klen = L;
    return nullity;
}

void orc_free(void *ptr)
{
    free(ptr);
}

/* ------------------------------------------------------------------ */
/* layout conversions (nmod_mat_poly_set_from.c:31-52,                 */
/* nmod_poly_mat_utils.c:185-210)                                      */
/* ------------------------------------------------------------------ */

int64_t orc_poly_mat_to_mat_poly(uint64_t *out, int64_t out_cap, const uint64_t *in, int64_t r, int64_t c,
                                 int64_t ld, int64_t len, int64_t order)
{
    const int64_t ne = r * c, K = order < len ? order : len;
    for (int64_t k = 0; k < out_cap; k++)
        for (int64_t e = 0; e < ne; e++)
            out[k * ne + e] = k < K ? in[e * ld + k] : 0;
    /* normalise: drop trailing zero coefficient matrices */
    int64_t L = K;
    while (L > 0)
    {
        int nz = 0;
        for (int64_t e = 0; e < ne && !nz; e++)
            nz = out[(L - 1) * ne + e] != 0;
        if (nz)
            break;
        L--;
    }
    return L;
}

void orc_mat_poly_to_poly_mat(uint64_t *out, int64_t out_cap, const uint64_t *in, int64_t r, int64_t c,
                              int64_t len, int64_t order)
{
    const int64_t ne = r * c, K = order < len ? order : len;
    for (int64_t e = 0; e < ne; e++)
        for (int64_t k = 0; k < out_cap; k++)
            out[e * out_cap + k] = k < K ? in[k * ne + e] : 0;
}

/* ------------------------------------------------------------------ */
/* truncated inverse and Dixon lifting (nmod_poly_mat_dixon.c)         */
/* ------------------------------------------------------------------ */

/* nmod_poly_mat_inv_trunc (nmod_poly_mat_dixon.c:32-80): S = A^-1 mod x^order from the
 * approximant basis of [A \\ -I] at order with shift [0, ..., 0, order, ..., order];
 * A invertible at x = 0 <=> the bottom-right block of the basis is the identity.
 * A: n x n, capacity alen; S: n x n, capacity order + 1.  Returns 1 (invertible) or 0. */
int orc_inv_trunc(uint64_t *S, const uint64_t *A, int64_t n, int64_t alen, int64_t order, uint64_t p,
                  int nthreads)
{
    const int64_t m = 2 * n, hl = alen > 0 ? alen : 1;
    uint64_t *H = (uint64_t *) calloc((size_t) (m * n * hl + 1), sizeof(uint64_t));
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            memcpy(H + (i * n + j) * hl, A + (i * n + j) * alen, sizeof(uint64_t) * (size_t) alen);
    for (int64_t i = n; i < m; i++)
        H[(i * n + (i - n)) * hl] = p - 1;
    int64_t *shift = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    for (int64_t i = 0; i < m; i++)
        shift[i] = i < n ? 0 : order;
    const int64_t cap = order + 1;
    uint64_t *T = (uint64_t *) calloc((size_t) (m * m * cap + 1), sizeof(uint64_t));
    orc_pmbasis(T, shift, H, m, n, hl, order, p, 32, nthreads);
    int is_inv = 1;
    for (int64_t i = 0; i < n && is_inv; i++)
        for (int64_t j = 0; j < n && is_inv; j++)
        {
            const uint64_t *e = T + ((n + i) * m + (n + j)) * cap;
            for (int64_t d = 0; d < cap && is_inv; d++)
                if (e[d] != ((i == j && d == 0) ? 1u : 0u))
                    is_inv = 0;
        }
    if (is_inv)
        for (int64_t i = 0; i < n; i++)
            for (int64_t j = 0; j < n; j++)
                memcpy(S + (i * n + j) * cap, T + ((n + i) * m + j) * cap, sizeof(uint64_t) * (size_t) cap);
    free(H); free(shift); free(T);
    return is_inv;
}

/* nmod_poly_mat_dixon (nmod_poly_mat_dixon.c:92-143): X with A X = B mod x^sigma by
 * x-adic lifting with the inverse mod x^order.  A: n x n (capacity alen), B: n x m
 * (capacity blen); X: n x m of capacity L * order, L = ceil(sigma / order), the sum of
 * the digits x^(l order) S_l.  Returns 1, or 0 when A is not invertible at x = 0. */
int orc_dixon(uint64_t *X, const uint64_t *A, const uint64_t *B, int64_t n, int64_t m, int64_t alen,
              int64_t blen, int64_t order, int64_t sigma, uint64_t p, int nthreads)
{
    const int64_t ccap = order + 1;
    uint64_t *Cinv = (uint64_t *) calloc((size_t) (n * n * ccap + 1), sizeof(uint64_t));
    if (!orc_inv_trunc(Cinv, A, n, alen, order, p, nthreads))
    {
        free(Cinv);
        return 0;
    }
    const int64_t L = (sigma + order - 1) / order, xcap = L * order;
    memset(X, 0, sizeof(uint64_t) * (size_t) (n * m * xcap));
    /* BB: the current residue, capacity bcap (grows to the largest length it reaches) */
    int64_t bcap = blen > 0 ? blen : 1;
    uint64_t *BB = pm_recap(B, n, m, blen, bcap);
    for (int64_t l = 0; l * order < sigma; l++)
    {
        /* S = C * BB mod x^order */
        const int64_t sl = ccap + bcap - 1;
        uint64_t *full = (uint64_t *) calloc((size_t) (n * m * sl + 1), sizeof(uint64_t));
        orc_poly_mat_mul(full, Cinv, BB, n, n, m, ccap, bcap, p, nthreads);
        uint64_t *S = (uint64_t *) calloc((size_t) (n * m * order + 1), sizeof(uint64_t));
        for (int64_t e = 0; e < n * m; e++)
            for (int64_t d = 0; d < order && d < sl; d++)
                S[e * order + d] = full[e * sl + d];
        free(full);
        /* X += x^(l order) S */
        for (int64_t e = 0; e < n * m; e++)
            for (int64_t d = 0; d < order; d++)
                X[e * xcap + l * order + d] = S[e * order + d];
        /* BB = (BB - A S) div x^order */
        const int64_t tl = alen + order - 1;
        uint64_t *AS = (uint64_t *) calloc((size_t) (n * m * tl + 1), sizeof(uint64_t));
        orc_poly_mat_mul(AS, A, S, n, n, m, alen, order, p, nthreads);
        const int64_t ncap = (bcap > tl ? bcap : tl) - order > 0 ? (bcap > tl ? bcap : tl) - order : 1;
        uint64_t *NB = (uint64_t *) calloc((size_t) (n * m * ncap + 1), sizeof(uint64_t));
        for (int64_t e = 0; e < n * m; e++)
            for (int64_t d = 0; d < ncap; d++)
            {
                const int64_t k = d + order;
                const uint64_t b = k < bcap ? BB[e * bcap + k] : 0;
                const uint64_t a = k < tl ? AS[e * tl + k] : 0;
                NB[e * ncap + d] = b >= a ? b - a : b + p - a;
            }
        free(AS); free(S); free(BB);
        BB = NB;
        bcap = ncap;
    }
    free(BB); free(Cinv);
    return 1;
}

/* ------------------------------------------------------------------ */
/* shifted Popov approximant basis: popov_pmbasis                      */
/* (ntl-extras/mat_lzz_pX_extra/src/mat_lzz_pX_pmbasis.cpp:1527-1557;  */
/* the TODO of flint-extras nmod_poly_mat_approximant.h:337-348)       */
/* ------------------------------------------------------------------ */

/* the t-row leading matrix of P (m x m, capacity cap): row i holds the coefficients of
 * degree rdeg_t(i) - t[j] of its entries (zero where that degree is out of range) */
static void row_leading_matrix(uint64_t *lm, const uint64_t *P, int64_t m, int64_t cap, const int64_t *t)
{
    for (int64_t i = 0; i < m; i++)
    {
        int64_t rd = INT64_MIN;
        for (int64_t j = 0; j < m; j++)
        {
            const int64_t d = poly_deg(P + (i * m + j) * cap, cap);
            if (d >= 0 && d + t[j] > rd)
                rd = d + t[j];
        }
        for (int64_t j = 0; j < m; j++)
        {
            const int64_t k = rd == INT64_MIN ? -1 : rd - t[j];
            lm[i * m + j] = (k >= 0 && k < cap) ? P[(i * m + j) * cap + k] : 0;
        }
    }
}

int64_t orc_popov_pmbasis(uint64_t *appbas, int64_t *shift, const uint64_t *F, int64_t m, int64_t n,
                          int64_t flen, int64_t order, uint64_t p, int nthreads)
{
    const int64_t cap = order + 1;
    /* first call: the s-row degree */
    int64_t *rdeg = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    int64_t *pshift = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    int64_t *t = (int64_t *) malloc(sizeof(int64_t) * (size_t) m);
    memcpy(rdeg, shift, sizeof(int64_t) * (size_t) m);
    orc_pmbasis(appbas, rdeg, F, m, n, flen, order, p, 32, nthreads);
    /* second call with shift s - rdeg_s = minus the pivot degrees */
    for (int64_t i = 0; i < m; i++)
    {
        pshift[i] = shift[i] - rdeg[i];
        t[i] = pshift[i];
        shift[i] = rdeg[i];
    }
    orc_pmbasis(appbas, pshift, F, m, n, flen, order, p, 32, nthreads);
    /* appbas <- lmat^-1 appbas, lmat its t-row leading matrix */
    uint64_t *aug = (uint64_t *) calloc((size_t) (m * 2 * m), sizeof(uint64_t));
    uint64_t *lm = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m));
    row_leading_matrix(lm, appbas, m, cap, t);
    for (int64_t i = 0; i < m; i++)
    {
        for (int64_t j = 0; j < m; j++)
            aug[i * 2 * m + j] = lm[i * m + j];
        aug[i * 2 * m + m + i] = 1;
    }
    const int64_t rk = orc_nmod_mat_rref(aug, m, 2 * m, p);
    int64_t L = 0;
    if (rk == m)
    {
        uint64_t *inv = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * m));
        for (int64_t i = 0; i < m; i++)
            for (int64_t j = 0; j < m; j++)
                inv[i * m + j] = aug[i * 2 * m + m + j];
        uint64_t *out = (uint64_t *) calloc((size_t) (m * m * cap), sizeof(uint64_t));
        uint64_t *col = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) m);
        for (int64_t j = 0; j < m; j++)
            for (int64_t d = 0; d < cap; d++)
            {
                for (int64_t k = 0; k < m; k++)
                    col[k] = appbas[(k * m + j) * cap + d];
                for (int64_t i = 0; i < m; i++)
                {
                    u128 acc = 0;
                    for (int64_t k = 0; k < m; k++)
                        acc += (u128) inv[i * m + k] * col[k];
                    out[(i * m + j) * cap + d] = (uint64_t) (acc % p);
                }
            }
        memcpy(appbas, out, sizeof(uint64_t) * (size_t) (m * m * cap));
        free(out); free(col); free(inv);
        L = orc_pm_max_length(appbas, m, m, cap);
    }
    else
        L = -1;    /* cannot happen for an approximant basis: its leading matrix is invertible */
    free(aug); free(lm); free(rdeg); free(pshift); free(t);
    return L;
}

/* ------------------------------------------------------------------ */
/* nmod_poly_mat_kernel_via_approx (kernel.c:146-227) and the          */
/* orientation interface nmod_poly_mat_kernel (kernel.c:26-144)        */
/* ------------------------------------------------------------------ */

int64_t orc_kernel_via_approx(uint64_t **ker, int64_t *klen, int64_t *pivind, int64_t *shift,
                              const uint64_t *pmat, int64_t m, int64_t n, int64_t plen, uint64_t p,
                              int nthreads)
{
    const int64_t cap0 = plen > 0 ? plen : 1;
    const int64_t d = orc_pm_max_length(pmat, m, n, cap0) - 1;
    *klen = 1;
    if (d == -1)
    {
        uint64_t *K = (uint64_t *) calloc((size_t) (m * m + 1), sizeof(uint64_t));
        for (int64_t i = 0; i < m; i++) { K[i * m + i] = 1; pivind[i] = i; }
        *ker = K;
        return m;
    }
    if (m == 1)
    {
        *ker = (uint64_t *) calloc((size_t) (m * m + 1), sizeof(uint64_t));
        return 0;
    }
    if (m <= n)
    {
        /* full row rank of the constant coefficient => empty kernel (:171-184) */
        uint64_t *c0 = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * n));
        for (int64_t e = 0; e < m * n; e++)
            c0[e] = pmat[e * cap0];
        const int64_t r = orc_nmod_mat_rref(c0, m, n, p);
        free(c0);
        if (r == m)
        {
            *ker = (uint64_t *) calloc((size_t) (m * m + 1), sizeof(uint64_t));
            return 0;
        }
    }
    int64_t mn = shift[0], amp = shift[0];
    for (int64_t i = 0; i < m; i++)
    {
        const int64_t s = shift[i];
        pivind[i] = s;
        if (s < mn) mn = s;
        else if (s > amp) amp = s;
    }
    amp -= mn;
    const int64_t order = (m < n ? m : n) * d + amp + d + 1;
    const int64_t cap = order + 1;
    uint64_t *K = (uint64_t *) calloc((size_t) (m * m * cap + 1), sizeof(uint64_t));
    orc_pmbasis(K, pivind, pmat, m, n, cap0, order, p, 32, nthreads);
    int64_t nullity = 0;
    uint64_t *tmp = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (m * cap));
    for (int64_t i = 0; i < m; i++)
    {
        if (pivind[i] - shift[i] + amp < order - d)
        {
            shift[nullity] = pivind[i];
            pivind[nullity] = i;
            /* swap rows nullity and i */
            memcpy(tmp, K + nullity * m * cap, sizeof(uint64_t) * (size_t) (m * cap));
            memcpy(K + nullity * m * cap, K + i * m * cap, sizeof(uint64_t) * (size_t) (m * cap));
            memcpy(K + i * m * cap, tmp, sizeof(uint64_t) * (size_t) (m * cap));
            nullity++;
        }
    }
    free(tmp);
    /* kernel rows, trimmed; other rows zero */
    const int64_t L0 = orc_pm_max_length(K, nullity, m, cap);
    const int64_t L = L0 > 0 ? L0 : 1;
    uint64_t *out = (uint64_t *) calloc((size_t) (m * m * L + 1), sizeof(uint64_t));
    for (int64_t e = 0; e < nullity * m; e++)
        memcpy(out + e * L, K + e * cap, sizeof(uint64_t) * (size_t) L);
    free(K);
    *ker = out;
    *klen = L;
    return nullity;
}

/* entry (i, j) of an r x c matrix (capacity cap) -> Q[(j, i)] */
static uint64_t *pm_transpose(const uint64_t *P, int64_t r, int64_t c, int64_t cap)
{
    uint64_t *Q = (uint64_t *) calloc((size_t) (r * c * cap + 1), sizeof(uint64_t));
    for (int64_t i = 0; i < r; i++)
        for (int64_t j = 0; j < c; j++)
            memcpy(Q + (j * r + i) * cap, P + (i * c + j) * cap, sizeof(uint64_t) * (size_t) cap);
    return Q;
}

/* nmod_poly_mat_kernel (kernel.c:26-144), form ORD_WEAK_POPOV, orientation orient
 * (COL_UPPER 0, COL_LOWER 1, ROW_UPPER 2, ROW_LOWER 3).  pmat: r x c, capacity plen.
 * Left kernels (ROW_*): *ker is r x r with the basis in its first nullity rows; right
 * kernels (COL_*): *ker is c x c with the basis in its first nullity columns.  shift:
 * NULL for the default (row / column degrees, zero for zero rows / columns), else
 * in/out as in the reference.  Returns the nullity. */
int64_t orc_kernel(uint64_t **ker, int64_t *klen, int64_t *pivind, int64_t *shift, const uint64_t *pmat,
                   int64_t r, int64_t c, int64_t plen, uint64_t p, int orient, int nthreads)
{
    const int left = orient == 2 || orient == 3;
    const int64_t m = left ? r : c, n = left ? c : r, cap0 = plen > 0 ? plen : 1;
    int64_t *sh = (int64_t *) malloc(sizeof(int64_t) * (size_t) (m > 0 ? m : 1));
    if (shift)
        memcpy(sh, shift, sizeof(int64_t) * (size_t) m);
    else
        for (int64_t i = 0; i < m; i++)
        {
            int64_t mx = 0;
            for (int64_t j = 0; j < n; j++)
            {
                const uint64_t *e = left ? pmat + (i * c + j) * cap0 : pmat + (j * c + i) * cap0;
                const int64_t dg = poly_deg(e, cap0);
                if (dg > mx) mx = dg;
            }
            sh[i] = mx;
        }
    /* the ROW_LOWER problem: transposed for right kernels, rows reversed for *_UPPER / COL_LOWER */
    uint64_t *M = left ? pm_recap(pmat, r, c, cap0, cap0) : pm_transpose(pmat, r, c, cap0);
    const int rev = orient == 2 || orient == 1;
    if (rev)
    {
        for (int64_t i = 0; i < m / 2; i++)
        {
            for (int64_t j = 0; j < n * cap0; j++)
            {
                uint64_t t = M[i * n * cap0 + j];
                M[i * n * cap0 + j] = M[(m - 1 - i) * n * cap0 + j];
                M[(m - 1 - i) * n * cap0 + j] = t;
            }
            int64_t t = sh[i]; sh[i] = sh[m - 1 - i]; sh[m - 1 - i] = t;
        }
    }
    uint64_t *K = NULL;
    int64_t L = 1;
    const int64_t nul = orc_kernel_zls(&K, &L, pivind, sh, M, m, n, cap0, p, nthreads);
    free(M);
    if (rev && nul > 0)
    {
        /* reverse the kernel rows (and their shifts), then the columns; pivots mirrored */
        uint64_t *T = (uint64_t *) calloc((size_t) (m * m * L + 1), sizeof(uint64_t));
        for (int64_t i = 0; i < nul; i++)
            for (int64_t j = 0; j < m; j++)
                memcpy(T + (i * m + j) * L, K + ((nul - 1 - i) * m + (m - 1 - j)) * L, sizeof(uint64_t) * (size_t) L);
        free(K);
        K = T;
        for (int64_t i = 0; i < nul / 2; i++)
        {
            int64_t t = sh[i]; sh[i] = sh[nul - 1 - i]; sh[nul - 1 - i] = t;
            const int64_t a = m - 1 - pivind[i];
            pivind[i] = m - 1 - pivind[nul - 1 - i];
            pivind[nul - 1 - i] = a;
        }
        if (nul % 2)
            pivind[nul / 2] = m - 1 - pivind[nul / 2];
    }
    if (!left)
    {
        uint64_t *T = pm_transpose(K, m, m, L);
        free(K);
        K = T;
    }
    if (shift)
        memcpy(shift, sh, sizeof(int64_t) * (size_t) m);
    free(sh);
    *ker = K;
    *klen = L;
    return nul;
}
