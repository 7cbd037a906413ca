// leaf64.cuh -- the mbasis leaf for word-size primes of any size (uint64 residues,
// Montgomery arithmetic with R = 2^64) and for matrices beyond the 64 x 64 of the
// 32-bit leaves.
#pragma once
#include "pmlg_internal.cuh"

namespace pmlg {

// largest m and n the 64-bit leaf (and so pmbasis) takes
constexpr int LEAF64_MAXDIM = 1024;

struct Leaf64Args
{
    const uint64_t *F;      // entry-major input, entry stride ldF, flen coefficients used
    int64_t ldF, flen;
    uint64_t *out;          // entry-major appbas, entry stride ldo (fully written)
    int64_t ldo;
    uint64_t *R;            // [order][m][n] scratch ([2 order] stepped): the residual appbas * F mod x^order
    uint64_t *AB;           // [order + 1][m][m] scratch ([2 order + 1] stepped): appbas, coefficient-major
    uint64_t *E;            // [n][m] scratch in global memory, or null: in shared memory
    uint64_t *X;            // [m][min(m, n)] scratch in global memory, or null: in shared memory
    int64_t *shift;         // device, m entries: in and out
    unsigned long long *len_out;   // device: appbas' length
    // the stepped leaf (one launch per phase of every step) keeps its state in global memory
    uint64_t *Xg;           // [m][min(m, n)]: X of the current step, Montgomery form
    long long *sh;          // [m]: the shifts
    int *st;                // [16 + 3m]: step state, then the pivot rows, the non-pivot rows, the row offsets
    int m, n, order;
    uint64_t p;
    uint64_t pneg;          // -p^-1 mod 2^64 (p odd)
    uint64_t r1, r2;        // 2^64 mod p and 2^128 mod p
    int two;                // p = 2: plain bit arithmetic instead of Montgomery
};

// bytes of each global scratch buffer of one leaf; E and X are 0 when they live in
// shared memory.  stepped: the leaf runs as two launches per order step (from 24 rows up)
struct Leaf64Sizes
{
    size_t R, AB, E, X, sh, st;
    bool stepped;
};
Leaf64Sizes leaf64_sizes(int m, int n, int order);

// their sum, each buffer rounded up to 256 bytes (the pmbasis arena's alignment)
size_t leaf64_scratch_bytes(int m, int n, int order);

// fills the modulus fields of the arguments (p prime, p >= 2)
void leaf64_set_modulus(Leaf64Args &a, uint64_t p);

// launches the leaf (one CTA, or the stepped launches), stream-ordered
int leaf64_launch(pmlg_ctx *ctx, const Leaf64Args &a, cudaStream_t st);

}  // namespace pmlg
