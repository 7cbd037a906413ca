// pointwise.cuh -- batched matrix products modulo an NTT prime at the
// evaluation points (the one dense contraction of the pipeline).
#pragma once
#include "pmlg_internal.cuh"

namespace pmlg {

// Element (pt, i, j) of an operand lives at
//   base + (pt / pt_tile) * s_tile + (i * ld + j) * s_e + (pt % pt_tile) * s_p
// which covers both the point-tiled layout written by the NTT kernels
// (pt_tile = 4, s_e = 4, s_p = 1) and plain batch-major matrices
// (pt_tile = 1, s_tile = r*k, s_e = 1, s_p = 0).
struct PwOperand
{
    const uint32_t *base;
    int64_t s_tile;
    int64_t ld;
};

struct PwArgs
{
    PwOperand A, B;
    uint32_t *C;
    int64_t s_tile_c, ldc;
    int pt_tile, s_e, s_p;
    int64_t npts;
    int r, k, c;        // block shape, each <= 64
    uint32_t q, r32, r32q, oneq;
    uint32_t scale, scaleq;   // every product is multiplied by scale (N^-1 ahead of an inverse NTT)
    uint32_t w8[7];     // scale * 2^(8s) mod q for the limb recombination
    uint32_t wd[4][3];  // scale * 2^(8i + 10j) mod q for the FP16-digit recombination
    uint64_t negoff;    // multiple of q >= 2^56, makes signed digit sums non-negative
    int accumulate;     // C += A*B instead of C = A*B
    int lmt;            // FP16 form: blocks of 2^lmt >= r, k, c; 64 >> lmt points share one MMA problem
    int *err;           // device error word (bounded waits that gave up), may be null
};

// Launches the chosen form over all points; blocks larger than 64 are split
// by the caller.
int pointwise_launch(pmlg_ctx *ctx, const PwArgs &a, int form, cudaStream_t st);

// Fills the modulus-dependent fields of PwArgs; the products come out
// multiplied by `scale` (1 for plain matrix products).
void pointwise_set_modulus(PwArgs &a, uint32_t q, uint32_t scale = 1);

// Products with r, k, c of any size: splits into 64 x 64 blocks and
// accumulates over the inner blocks.
int pointwise_blocked(pmlg_ctx *ctx, PwArgs a, int64_t r, int64_t k, int64_t c, int form,
                      cudaStream_t st);

// Shape class of the form tuner: r, k, c (each <= 64) and npts rounded up to a power of two.
uint64_t tune_key(int r, int k, int c, int64_t npts);

}  // namespace pmlg
