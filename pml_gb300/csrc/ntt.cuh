// ntt.cuh -- forward / inverse number-theoretic transforms over 30-bit primes.
#pragma once
#include "pmlg_internal.cuh"

namespace pmlg {

// Largest transform handled by one CTA (16 residues per thread, 1024 threads).
constexpr int kMaxLgN = 14;
constexpr int kMinLgN = 4;

// Device view of one NttTable, for one direction.
struct NttDev
{
    const uint2 *w;      // group twiddle table of the direction (layout: NttTable)
    uint32_t q, ninv, ninvq, r32, r32q, oneq;
    uint32_t c16[8], c16q[8];   // (forward or inverse) sixteenth roots of unity
};

inline NttDev ntt_dev(const NttTable *t, bool inverse)
{
    NttDev d;
    d.w = inverse ? t->d_iw : t->d_w;
    d.q = t->q; d.ninv = t->ninv; d.ninvq = t->ninvq;
    d.r32 = t->r32; d.r32q = t->r32q; d.oneq = t->oneq;
    for (int j = 0; j < 8; j++) {
        d.c16[j] = inverse ? t->ic16[j] : t->c16[j];
        d.c16q[j] = inverse ? t->ic16q[j] : t->c16q[j];
    }
    return d;
}

// Evaluations are stored "point-tiled": for prime j, point t and matrix entry e,
//   E[j * prime_stride + (t / T) * tile_stride + e * T + (t % T)],  T = kPtTile,
// tile_stride = T * (number of entries), so that the T consecutive points of
// one entry are one 16-byte word (T = 4) and all entries of a tile are
// contiguous.  Point t holds the evaluation at w^bitrev(t).  The pointwise
// kernels read two points of an entry in one 8-byte load.  Measured on GB300
// for the 64x64 product at length 4096: T = 8 made the forward NTT 5 us faster
// and the pointwise products 27 us slower; T = 16 is worse still.
#ifndef PMLG_PT_TILE
#define PMLG_PT_TILE 4
#endif
constexpr int kPtTile = PMLG_PT_TILE;
static_assert(kPtTile == 4 || kPtTile == 8 || kPtTile == 16, "point tile");

struct NttFwdArgs
{
    const uint64_t *in;     // entry e starts at in + e * in_ld + in_off
    int64_t in_ld, in_off, L;   // L coefficients are read, the rest is zero
    int64_t nent;
    uint32_t *out;
    int64_t prime_stride, tile_stride;
    int lg, t, reduce;      // reduce: inputs are < 2^64 and need reduction mod q
    int use_tma;            // N >= 4096: evaluations leave through TMA tensor stores (set by ntt_forward)
    NttDev tab[kMaxPrimes];
};

struct NttInvArgs
{
    const uint32_t *in;     // point-tiled evaluations
    int64_t prime_stride, tile_stride;
    int64_t nent;
    int64_t lo, cnt;        // coefficients [lo, lo + cnt) of the length-N cyclic result
    // direct output (p is the NTT prime): out64[e * out_ld + d], d < out_cap, zero for d >= cnt
    uint64_t *out64;
    int64_t out_ld, out_cap;
    // CRT output (otherwise): res32[(j * nent + e) * cnt + d]
    uint32_t *res32;
    int lg, t, direct;
    int *err;               // device error word (a bounded wait gave up); set by ntt_inverse
    NttDev tab[kMaxPrimes];
};

int ntt_forward(pmlg_ctx *ctx, const NttFwdArgs &a, cudaStream_t st);
int ntt_inverse(pmlg_ctx *ctx, const NttInvArgs &a, cudaStream_t st);

// out64[e * out_ld + d] = CRT(res32[(j * nent + e) * cnt + d], j < t) mod p for
// d < cnt; zero for cnt <= d < out_cap.
int crt_combine(pmlg_ctx *ctx, const CrtPlan &plan, const uint32_t *res32, int64_t nent,
                int64_t cnt, uint64_t *out64, int64_t out_ld, int64_t out_cap, cudaStream_t st);

}  // namespace pmlg
