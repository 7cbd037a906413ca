// pmlg_internal.cuh -- shared device arithmetic, context and launch helpers.
//
// Arithmetic conventions
//   * Every internal transform works modulo a word prime q < 2^30 that has a
//     primitive 2^e-th root of unity (an "NTT prime"), on uint32 residues.
//     Lazy butterflies keep values in [0, 2q) or [0, 4q); 4q < 2^32.
//   * Multiplication by a fixed operand w uses Shoup's method with the
//     precomputed quotient w' = floor(w * 2^32 / q), computed with exact 64-bit
//     integer division on the host (no floating point anywhere).
//   * Word-size moduli p that are not such a prime (and p >= 2^30) are handled by
//     computing the exact integer result modulo several NTT primes and
//     reconstructing it by CRT, then reducing mod p.
#pragma once

#include <cstdint>
#include <cstddef>
#include <map>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/pmlg.h"

namespace pmlg {

// ---------------------------------------------------------------------------
// device arithmetic
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ uint32_t shoup_mul(uint32_t x, uint32_t w, uint32_t wq, uint32_t q)
{
    // x < 2^32, w < q < 2^31: returns x*w mod q in [0, 2q)
#ifdef __CUDA_ARCH__
    uint32_t hi = __umulhi(x, wq);
#else
    uint32_t hi = (uint32_t)(((uint64_t)x * wq) >> 32);
#endif
    return x * w - hi * q;
}

__host__ __device__ __forceinline__ uint32_t reduce_once(uint32_t x, uint32_t q)
{
    return x >= q ? x - q : x;
}

// Reduction of a 64-bit value x = hi*2^32 + lo modulo a prime q < 2^30, using
// r32 = 2^32 mod q with its Shoup quotient, and oneq = floor(2^32 / q) (the
// Shoup quotient of w = 1).  Both partial results lie in [0, 2q).
__host__ __device__ __forceinline__ uint32_t mod64_q(uint64_t x, uint32_t q, uint32_t r32,
                                                     uint32_t r32q, uint32_t oneq)
{
    uint32_t hi = (uint32_t)(x >> 32), lo = (uint32_t)x;
    uint32_t t = shoup_mul(hi, r32, r32q, q);       // hi*2^32 mod q, in [0, 2q)
    uint32_t l = shoup_mul(lo, 1u, oneq, q);        // lo mod q, in [0, 2q)
    uint32_t s = t + l;                              // < 4q < 2^32
    s = s >= 2 * q ? s - 2 * q : s;
    s = s >= q ? s - q : s;
    return s;
}

// ---------------------------------------------------------------------------
// NTT tables
// ---------------------------------------------------------------------------

// Twiddles for one (prime, N), w a primitive N-th root of unity mod q.
// The radix-16 groups of the NTT need, for a group whose sub-transforms are
// spaced L = 2^lls apart (span 16L), the factors w_span^(off * bitrev4(m)) for
// off < L and m = 1..15.  They are stored per group size, coalesced over off:
//   d_w[15 (2^lls - 1) + (m - 1) 2^lls + off] = {w^(off bitrev4(m) N / 16L), quotient}
// (d_iw: the same with w^-1), lls = 0 .. lg-4, fewer than 2N entries each.
// c16 holds the sixteenth roots w^(jN/16), j < 8, of the butterflies.
struct NttTable
{
    uint32_t q;
    int lg;            // N = 2^lg
    uint2 *d_w;        // forward group twiddles
    uint2 *d_iw;       // inverse group twiddles
    uint32_t c16[8], c16q[8];      // w^(jN/16) and quotients
    uint32_t ic16[8], ic16q[8];    // w^(-jN/16) and quotients
    uint32_t ninv, ninvq;    // N^{-1} mod q and quotient
    uint32_t r32, r32q;      // 2^32 mod q and quotient
    uint32_t oneq;           // floor(2^32 / q)
};

// CRT plan: the exact integer result is recovered from t residues modulo NTT
// primes by Garner's mixed radix form and reduced mod the target p.
constexpr int kMaxPrimes = 6;

struct CrtPlan
{
    int direct;                    // 1: p itself is the (single) NTT prime, no CRT
    int t;                         // number of primes
    uint32_t q[kMaxPrimes];
    // garner[j][l] = q_l mod q_j (l < j), ginv[j] = (q_0..q_{j-1})^{-1} mod q_j
    uint32_t qmod[kMaxPrimes][kMaxPrimes];
    uint32_t qmodq[kMaxPrimes][kMaxPrimes];
    uint32_t ginv[kMaxPrimes], ginvq[kMaxPrimes];
    // for the final Horner mod p: q_l mod p and its 64-bit Shoup quotient
    // floor(qp * 2^64 / p), and floor(2^64 / p) to reduce residues below 2^30
    uint64_t qp[kMaxPrimes], qpq[kMaxPrimes];
    uint64_t onepq;
    uint64_t p;
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------

struct Workspace
{
    void *ptr = nullptr;
    size_t bytes = 0;
};

// one profiled kernel launch: CUDA events recorded on the launch stream
struct ProfRecord
{
    const char *name;
    cudaEvent_t beg, end;
};

}  // namespace pmlg

struct pmlg_ctx
{
    int device = 0;
    int form = PMLG_FORM_AUTO;
    int64_t leaf_order = 0;        // 0 = autotuned default
    int sm_count = 0;
    pmlg::Workspace ws;            // device scratch, grown on demand
    pmlg::Workspace ws_aux;        // second scratch (host-buffer copies, reductions)
    pmlg::Workspace ws_pm;         // pmbasis recursion arena
    void *pinned = nullptr;        // pinned staging for host-buffer entry points
    size_t pinned_bytes = 0;
    unsigned long long launches = 0;   // kernels launched through this context
    int *d_err = nullptr;              // device error word: a bounded wait gave up
    // streams and events of the batched products (created on first use)
    static constexpr int kBatchStreams = 8;
    cudaStream_t bstream[kBatchStreams] = {};
    cudaEvent_t bevent[kBatchStreams + 1] = {};
    // events of the host-buffer product's copy/compute pipeline
    static constexpr int kHostEvents = 40;
    cudaEvent_t hevent[kHostEvents] = {};
    pmlg::Workspace ws_batch;      // per-stream scratch of the batched products
    // cached NTT tables
    static constexpr int kMaxTables = 256;
    pmlg::NttTable tables[kMaxTables];
    int ntables = 0;
    char last_error[256] = {0};
    // per-kernel timing (pmlg_ctx_set_profiling): events around every launch
    int profiling = 0;
    std::vector<pmlg::ProfRecord> prof;
    std::vector<cudaEvent_t> event_pool;
    // PMLG_FORM_AUTO: pointwise form chosen per shape class by measurement
    int tuning = 1;                          // 0: AUTO takes the FP16 form unmeasured
    std::map<uint64_t, int> tuned;           // shape class -> fastest form measured
    // batched products: a repeated batch is captured into a CUDA graph and replayed
    struct BatchGraph
    {
        uint64_t key = 0;
        std::vector<uint64_t> sig;           // the full batch description the key hashes
        cudaGraphExec_t exec = nullptr;
        unsigned long long launches = 0;
    };
    static constexpr int kBatchGraphs = 4;
    int batch_graphs = 1;                    // 0: every batch launches its kernels directly
    BatchGraph bgraph[kBatchGraphs];
    int bgraph_next = 0;
    uint64_t batch_seen = 0;                 // key of the last batch launched directly
    std::vector<uint64_t> batch_seen_sig;    // and its full description
};

namespace pmlg {

// status helpers
#define PMLG_CUDA_TRY(expr)                                                   \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) {                                              \
            pmlg::set_error(ctx, "%s: %s", #expr, cudaGetErrorString(_e));    \
            return PMLG_ECUDA;                                                \
        }                                                                     \
    } while (0)

#define PMLG_TRY(expr)                                                        \
    do {                                                                      \
        int _s = (expr);                                                      \
        if (_s != PMLG_OK) return _s;                                         \
    } while (0)

void set_error(pmlg_ctx *ctx, const char *fmt, ...);

// Waits for the stream, then reads and clears the device error word: PMLG_ETIMEOUT
// when a bounded device wait of an earlier kernel on this context gave up.
int device_status(pmlg_ctx *ctx, cudaStream_t st);

// scalar host arithmetic
uint64_t h_mulmod(uint64_t a, uint64_t b, uint64_t p);
uint64_t h_powmod(uint64_t a, uint64_t e, uint64_t p);
uint64_t h_invmod(uint64_t a, uint64_t p);
bool h_is_prime(uint64_t n);
inline uint32_t h_shoup_q(uint32_t w, uint32_t q) { return (uint32_t)(((uint64_t)w << 32) / q); }

// table access (built on demand, cached in the context)
int get_table(pmlg_ctx *ctx, uint32_t q, int lg, const NttTable **out);

// prime selection: direct when p is an NTT prime < 2^30 with 2^lg | p-1,
// otherwise enough CRT primes to hold k * min(len1,len2) * (p-1)^2.
int make_plan(pmlg_ctx *ctx, uint64_t p, int lg, int64_t inner, int64_t minlen, CrtPlan *plan);

// scratch memory
int ws_reserve(pmlg_ctx *ctx, Workspace *ws, size_t bytes);

// max length (last nonzero coefficient + 1) over the entries of a device
// polynomial matrix; synchronises the stream
int device_max_length(pmlg_ctx *ctx, const uint64_t *P, int64_t nent, int64_t ld, int64_t len,
                      unsigned long long *d_tmp, int64_t *out, cudaStream_t st);

inline void count_launch(pmlg_ctx *ctx, unsigned n = 1) { ctx->launches += n; }

// Kernel-timing hooks: no-ops unless profiling is on.  prof_begin records an
// event on the launch stream before the kernel, prof_end one after it.
void prof_begin(pmlg_ctx *ctx, const char *name, cudaStream_t st);
void prof_end(pmlg_ctx *ctx, cudaStream_t st);

}  // namespace pmlg
