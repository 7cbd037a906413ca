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
    uint64_t *R;            // [order][m][n] scratch: the residual appbas * F mod x^order
    uint64_t *AB;           // [order + 1][m][m] scratch: appbas, coefficient-major
    uint64_t *E;            // [n][m] scratch in global memory, or null: in shared memory
    uint64_t *X;            // [m][min(m, n)] scratch in global memory, or null: in shared memory
    int64_t *shift;         // device, m entries: in and out
    unsigned long long *len_out;   // device: appbas' length
    // the stepped leaf (one launch per phase of every step) keeps its state in global memory
    uint64_t *Xg;           // [m][min(m, n)]: X of the current step, Montgomery form
    long long *sh;          // [m]: the shifts
    int *st;                // [16 + 2m]: step state, then the pivot rows and the non-pivot rows
    int m, n, order;
    uint64_t p;
    uint64_t pneg;          // -p^-1 mod 2^64 (p odd)
    uint64_t r1, r2;        // 2^64 mod p and 2^128 mod p
    int two;                // p = 2: plain bit arithmetic instead of Montgomery
};

// bytes of global scratch the leaf needs (R, AB, and E / X when they do not fit in
// shared memory); sets *e_shared / *x_shared to whether they go to shared memory
size_t leaf64_scratch_bytes(int m, int n, int order, bool *e_shared, bool *x_shared);

// fills the modulus fields of the arguments (p prime, p >= 2)
void leaf64_set_modulus(Leaf64Args &a, uint64_t p);

// launches the leaf: one CTA, stream-ordered
int leaf64_launch(pmlg_ctx *ctx, const Leaf64Args &a, cudaStream_t st);

}  // namespace pmlg
