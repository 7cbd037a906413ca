// polymat.cu -- nmod_poly_mat_multiply / mulmid on the GPU:
// forward NTT of every entry -> pointwise matrix products at the N points ->
// inverse NTT (+ CRT when the modulus is not an NTT prime).
//
// The reference evaluates at a geometric progression (FLINT
// _nmod_poly_evaluate_geometric_nmod_vec_fast_precomp, mul_geometric.c:78,89)
// and interpolates (mul_geometric.c:104); evaluating at 2^lg-th roots of unity
// gives the same unique product mod p.  Middle products use the cyclic
// wrap-around of a length-N transform: with N >= nhi and N >= len1+len2-1-nlo,
// the coefficients [nlo, nhi) of the cyclic product equal those of the full one.
#include "polymat.cuh"
#include "ntt.cuh"
#include "pointwise.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace pmlg {

int lg_for(int64_t n)
{
    int lg = kMinLgN;
    while ((1ll << lg) < n) lg++;
    return lg;
}

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t product_scratch_bytes(const ProductJob &j, const CrtPlan &plan)
{
    const size_t N = (size_t)1 << j.lg, t = plan.t;
    size_t b = 0;
    b += align256(t * N * j.r * j.k * 4);
    b += align256(t * N * j.k * j.c * 4);
    b += align256(t * N * j.r * j.c * 4);
    if (!plan.direct) b += align256(t * j.r * j.c * j.cnt * 4);
    return b;
}

// The scratch of a product: evaluations of A, B and C per prime (point-tiled),
// and the CRT residues when p is not the NTT prime.
struct ProductBufs
{
    uint32_t *EA, *EB, *EC, *R32;
    const NttTable *tabs[kMaxPrimes];
};

static int product_bufs(pmlg_ctx *ctx, const ProductJob &j, const CrtPlan &plan, void *scratch, ProductBufs &b)
{
    const int64_t N = 1ll << j.lg;
    const int t = plan.t;
    char *w = (char *)scratch;
    b.EA = (uint32_t *)w; w += align256((size_t)t * N * j.r * j.k * 4);
    b.EB = (uint32_t *)w; w += align256((size_t)t * N * j.k * j.c * 4);
    b.EC = (uint32_t *)w; w += align256((size_t)t * N * j.r * j.c * 4);
    b.R32 = plan.direct ? nullptr : (uint32_t *)w;
    for (int i = 0; i < t; i++) PMLG_TRY(get_table(ctx, plan.q[i], j.lg, &b.tabs[i]));
    return PMLG_OK;
}

// forward transforms of the entries [e0, e1) of A (which = 0) or B (which = 1)
static int product_forward(pmlg_ctx *ctx, const ProductJob &j, const CrtPlan &plan, const ProductBufs &b,
                           int which, int64_t e0, int64_t e1, cudaStream_t st)
{
    const int64_t N = 1ll << j.lg;
    if (e1 <= e0) return PMLG_OK;
    NttFwdArgs fa{};
    fa.lg = j.lg;
    fa.t = plan.t;
    fa.reduce = !plan.direct;
    for (int i = 0; i < plan.t; i++) fa.tab[i] = ntt_dev(b.tabs[i], false);
    if (which == 0) {
        const int64_t nA = j.r * j.k;
        fa.in = j.A + e0 * j.lda; fa.in_ld = j.lda; fa.in_off = j.a_off; fa.L = j.a_len; fa.nent = e1 - e0;
        fa.out = b.EA + e0 * kPtTile; fa.prime_stride = N * nA; fa.tile_stride = kPtTile * nA;
    } else {
        const int64_t nB = j.k * j.c;
        fa.in = j.B + e0 * j.ldb; fa.in_ld = j.ldb; fa.in_off = j.b_off; fa.L = j.b_len; fa.nent = e1 - e0;
        fa.out = b.EB + e0 * kPtTile; fa.prime_stride = N * nB; fa.tile_stride = kPtTile * nB;
    }
    return ntt_forward(ctx, fa, st);
}

// pointwise products of the rows [i0, i1) of A and C, one prime at a time (scaled by
// 1/N for the inverse transform)
static int product_pointwise(pmlg_ctx *ctx, const ProductJob &j, const CrtPlan &plan, const ProductBufs &b,
                             int64_t i0, int64_t i1, int form, cudaStream_t st)
{
    const int64_t N = 1ll << j.lg;
    const int64_t nA = j.r * j.k, nB = j.k * j.c, nC = j.r * j.c;
    if (i1 <= i0) return PMLG_OK;
    for (int i = 0; i < plan.t; i++) {
        PwArgs pa{};
        pa.A = {b.EA + (size_t)i * N * nA + i0 * j.k * kPtTile, kPtTile * nA, j.k};
        pa.B = {b.EB + (size_t)i * N * nB, kPtTile * nB, j.c};
        pa.C = b.EC + (size_t)i * N * nC + i0 * j.c * kPtTile;
        pa.s_tile_c = kPtTile * nC;
        pa.ldc = j.c;
        pa.pt_tile = kPtTile;
        pa.s_e = kPtTile;
        pa.s_p = 1;
        pa.npts = N;
        pa.accumulate = 0;
        pointwise_set_modulus(pa, plan.q[i], b.tabs[i]->ninv);   // the 1/N of the inverse transform
        PMLG_TRY(pointwise_blocked(ctx, pa, i1 - i0, j.k, j.c, form, st));
    }
    return PMLG_OK;
}

// inverse transforms of the output entries [e0, e1) (+ CRT when p is not the NTT prime)
static int product_inverse(pmlg_ctx *ctx, const ProductJob &j, const CrtPlan &plan, const ProductBufs &b,
                           int64_t e0, int64_t e1, cudaStream_t st)
{
    const int64_t N = 1ll << j.lg;
    const int64_t nC = j.r * j.c, ne = e1 - e0;
    if (ne <= 0) return PMLG_OK;
    NttInvArgs ia{};
    ia.in = b.EC + e0 * kPtTile; ia.prime_stride = N * nC; ia.tile_stride = kPtTile * nC; ia.nent = ne;
    ia.lo = j.lo; ia.cnt = j.cnt;
    ia.out64 = j.C + e0 * j.ldc; ia.out_ld = j.ldc; ia.out_cap = j.c_cap;
    ia.res32 = b.R32;
    ia.lg = j.lg; ia.t = plan.t; ia.direct = plan.direct;
    for (int i = 0; i < plan.t; i++) ia.tab[i] = ntt_dev(b.tabs[i], true);
    PMLG_TRY(ntt_inverse(ctx, ia, st));
    if (!plan.direct)
        PMLG_TRY(crt_combine(ctx, plan, b.R32, ne, j.cnt, j.C + e0 * j.ldc, j.ldc, j.c_cap, st));
    return PMLG_OK;
}

int product_run(pmlg_ctx *ctx, const ProductJob &j, const CrtPlan &plan, void *scratch, int form,
                cudaStream_t st, EvalCache *ca)
{
    ProductBufs b;
    PMLG_TRY(product_bufs(ctx, j, plan, scratch, b));
    const size_t need = (size_t)plan.t * ((size_t)1 << j.lg) * (size_t)(j.r * j.k);
    if (ca && ca->ea && need <= ca->words) {
        bool same = ca->valid && ca->lg == j.lg && ca->t == plan.t && ca->a == j.A && ca->r == j.r && ca->k == j.k && ca->lda == j.lda &&
                    ca->a_off == j.a_off && ca->a_len == j.a_len;
        for (int i = 0; same && i < plan.t; i++) same = ca->q[i] == plan.q[i];
        b.EA = ca->ea;
        if (!same) {
            ca->valid = false;
            PMLG_TRY(product_forward(ctx, j, plan, b, 0, 0, j.r * j.k, st));
            ca->valid = true;
            ca->lg = j.lg;
            ca->t = plan.t;
            for (int i = 0; i < plan.t; i++) ca->q[i] = plan.q[i];
            ca->a = j.A;
            ca->r = j.r;
            ca->k = j.k;
            ca->lda = j.lda;
            ca->a_off = j.a_off;
            ca->a_len = j.a_len;
        }
    } else {
        PMLG_TRY(product_forward(ctx, j, plan, b, 0, 0, j.r * j.k, st));
    }
    PMLG_TRY(product_forward(ctx, j, plan, b, 1, 0, j.k * j.c, st));
    PMLG_TRY(product_pointwise(ctx, j, plan, b, 0, j.r, form, st));
    return product_inverse(ctx, j, plan, b, 0, j.r * j.c, st);
}

int mulmid_prepare(ProductJob &j, int64_t len1, int64_t len2, int64_t nlo, int64_t nhi)
{
    int64_t a_len = len1 < nhi ? len1 : nhi;
    int64_t b_len = len2 < nhi ? len2 : nhi;
    int64_t a_off = 0, b_off = 0, lo = nlo;
    int64_t hi = nhi;
    if (hi > a_len + b_len - 1) hi = a_len + b_len - 1;
    if (a_len <= 0 || b_len <= 0 || hi <= lo) {
        j.cnt = 0;
        return 0;
    }
    // coefficients of B below lo - (a_len - 1) only reach product terms below lo
    int64_t sB = lo - (a_len - 1);
    if (sB > 0) { b_off += sB; b_len -= sB; lo -= sB; hi -= sB; }
    int64_t sA = lo - (b_len - 1);
    if (sA > 0) { a_off += sA; a_len -= sA; lo -= sA; hi -= sA; }
    j.a_off = a_off; j.a_len = a_len;
    j.b_off = b_off; j.b_len = b_len;
    j.lo = lo;
    j.cnt = hi - lo;
    int64_t need = hi;
    if (a_len + b_len - 1 - lo > need) need = a_len + b_len - 1 - lo;
    j.lg = lg_for(need);
    return j.lg;
}

// ---------------------------------------------------------------------------
// max length of a polynomial matrix (device), for the clamped lengths
// ---------------------------------------------------------------------------

__global__ void maxlen_kernel(const uint64_t *__restrict__ P, int64_t nent, int64_t ld, int64_t len,
                              unsigned long long *out)
{
    const int64_t total = nent * len;
    unsigned long long best = 0;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx / len, d = idx - e * len;
        if (P[e * ld + d] != 0 && (unsigned long long)(d + 1) > best) best = d + 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_down_sync(0xffffffffu, best, o);
        best = v > best ? v : best;
    }
    if ((threadIdx.x & 31) == 0 && best) atomicMax(out, best);
}

int device_max_length(pmlg_ctx *ctx, const uint64_t *P, int64_t nent, int64_t ld, int64_t len,
                      unsigned long long *d_tmp, int64_t *out, cudaStream_t st)
{
    PMLG_CUDA_TRY(cudaMemsetAsync(d_tmp, 0, sizeof(unsigned long long), st));
    if (nent > 0 && len > 0) {
        int64_t blocks = (nent * len + 255) / 256;
        if (blocks > (int64_t)ctx->sm_count * 8) blocks = (int64_t)ctx->sm_count * 8;
        prof_begin(ctx, "maxlen", st);
        maxlen_kernel<<<(unsigned)blocks, 256, 0, st>>>(P, nent, ld, len, d_tmp);
        prof_end(ctx, st);
        count_launch(ctx);
        PMLG_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long h = 0;
    PMLG_CUDA_TRY(cudaMemcpyAsync(&h, d_tmp, sizeof(h), cudaMemcpyDeviceToHost, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    *out = (int64_t)h;
    return PMLG_OK;
}

static bool overlaps(const void *a, size_t na, const void *b, size_t nb)
{
    const char *x = (const char *)a, *y = (const char *)b;
    return na && nb && x < y + nb && y < x + na;
}

// ---------------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------------

static int run_job_alloc(pmlg_ctx *ctx, const ProductJob &j, cudaStream_t st, EvalCache *ca = nullptr)
{
    CrtPlan plan;
    const int64_t minlen = j.a_len < j.b_len ? j.a_len : j.b_len;
    PMLG_TRY(make_plan(ctx, j.p, j.lg, j.k, minlen, &plan));
    PMLG_TRY(ws_reserve(ctx, &ctx->ws, product_scratch_bytes(j, plan)));
    return product_run(ctx, j, plan, ctx->ws.ptr, ctx->form, st, ca);
}

// the job of a full product C = A * B with coefficient-contiguous entries
static void full_product_job(ProductJob &j, uint64_t *C, const uint64_t *A, const uint64_t *B, int64_t r,
                             int64_t k, int64_t c, int64_t len1, int64_t len2, uint64_t p)
{
    const int64_t clen = len1 + len2 - 1;
    j = ProductJob{};
    j.r = r; j.k = k; j.c = c;
    j.A = A; j.lda = len1; j.a_off = 0; j.a_len = len1;
    j.B = B; j.ldb = len2; j.b_off = 0; j.b_len = len2;
    j.C = C; j.ldc = clen; j.c_cap = clen;
    j.lo = 0; j.cnt = clen;
    j.lg = lg_for(clen);
    j.p = p;
}

// the context's side streams and events (batched products, host-buffer pipelining)
static int ensure_side_streams(pmlg_ctx *ctx, int nstreams)
{
    for (int s = 0; s < nstreams; s++)
        if (!ctx->bstream[s]) PMLG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->bstream[s], cudaStreamNonBlocking));
    for (int s = 0; s <= pmlg_ctx::kBatchStreams; s++)
        if (!ctx->bevent[s]) PMLG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->bevent[s], cudaEventDisableTiming));
    for (int s = 0; s < pmlg_ctx::kHostEvents; s++)
        if (!ctx->hevent[s]) PMLG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->hevent[s], cudaEventDisableTiming));
    return PMLG_OK;
}

int poly_mat_mul_device(pmlg_ctx *ctx, uint64_t *C, const uint64_t *A, const uint64_t *B, int64_t r,
                        int64_t k, int64_t c, int64_t len1, int64_t len2, uint64_t p, cudaStream_t st,
                        EvalCache *ca)
{
    const int64_t clen = (len1 > 0 && len2 > 0) ? len1 + len2 - 1 : 0;
    if (r == 0 || c == 0 || clen == 0) return PMLG_OK;
    if (k == 0) {
        PMLG_CUDA_TRY(cudaMemsetAsync(C, 0, (size_t)(r * c * clen) * 8, st));
        return PMLG_OK;
    }
    ProductJob j;
    full_product_job(j, C, A, B, r, k, c, len1, len2, p);
    if (j.lg > kMaxLgN) {
        set_error(ctx, "product length %lld needs a transform beyond 2^%d", (long long)clen, kMaxLgN);
        return PMLG_ELEN;
    }
    return run_job_alloc(ctx, j, st, ca);
}

int poly_mat_mulmid_device(pmlg_ctx *ctx, uint64_t *res, const uint64_t *A, const uint64_t *B,
                           int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2, int64_t nlo,
                           int64_t nhi, uint64_t p, cudaStream_t st, EvalCache *ca)
{
    const int64_t cap = nhi - nlo;
    if (cap <= 0 || r == 0 || c == 0) return PMLG_OK;
    ProductJob j{};
    j.r = r; j.k = k; j.c = c;
    j.A = A; j.lda = len1;
    j.B = B; j.ldb = len2;
    j.C = res; j.ldc = cap; j.c_cap = cap;
    j.p = p;
    mulmid_prepare(j, k == 0 ? 0 : len1, len2, nlo, nhi);
    if (j.cnt <= 0) {
        PMLG_CUDA_TRY(cudaMemsetAsync(res, 0, (size_t)(r * c * cap) * 8, st));
        return PMLG_OK;
    }
    if (j.lg > kMaxLgN) {
        set_error(ctx, "middle product needs a transform beyond 2^%d", kMaxLgN);
        return PMLG_ELEN;
    }
    return run_job_alloc(ctx, j, st, ca);
}

static int check_common(pmlg_ctx *ctx, const void *C, const void *A, const void *B, int64_t r, int64_t k,
                        int64_t c, int64_t len1, int64_t len2, uint64_t p)
{
    if (!ctx) return PMLG_EINVAL;
    if (r < 0 || k < 0 || c < 0 || len1 < 0 || len2 < 0) return PMLG_EINVAL;
    if (p < 2) { set_error(ctx, "modulus must be >= 2"); return PMLG_EBADMOD; }
    if ((r * k * len1 > 0 && !A) || (k * c * len2 > 0 && !B) || (r * c > 0 && !C)) return PMLG_EINVAL;
    return PMLG_OK;
}

// host -> device copy on the stream (asynchronous when the source is pinned)
#ifndef PMLG_HOST_ROW_BLOCKS
#define PMLG_HOST_ROW_BLOCKS 4
#endif
#ifndef PMLG_HOST_2D
#define PMLG_HOST_2D 1      // host-buffer products with one NTT prime: blocks of C in both directions
#endif
#ifndef PMLG_HOST_BR
#define PMLG_HOST_BR 2      // row blocks of C (and A) in that pipeline
#endif
#ifndef PMLG_HOST_BC
#define PMLG_HOST_BC 3      // column blocks of C (and B)
#endif
// row blocks of the host-buffer product's pipeline (events used: 2 + 4 + 2 * blocks)
constexpr int kHostRowBlocks = PMLG_HOST_ROW_BLOCKS;
static_assert(2 + 4 + 2 * kHostRowBlocks <= pmlg_ctx::kHostEvents, "host pipeline events");
constexpr int kHostBR = PMLG_HOST_BR, kHostBC = PMLG_HOST_BC;
static_assert(kHostBR >= 1 && kHostBC >= 1 && 2 + kHostBR + kHostBC + kHostBR * kHostBC <= pmlg_ctx::kHostEvents,
              "host pipeline events");

static int h2d(pmlg_ctx *ctx, void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    if (!bytes) return PMLG_OK;
    PMLG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return PMLG_OK;
}

}  // namespace pmlg

using namespace pmlg;

extern "C" {

PMLG_API int pmlg_poly_mat_mul(pmlg_ctx *ctx, uint64_t *C, const uint64_t *A, const uint64_t *B,
                               int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                               uint64_t p, void *stream)
{
    PMLG_TRY(check_common(ctx, C, A, B, r, k, c, len1, len2, p));
    const int64_t clen = (len1 > 0 && len2 > 0) ? len1 + len2 - 1 : 0;
    if (overlaps(C, (size_t)(r * c * clen) * 8, A, (size_t)(r * k * len1) * 8) ||
        overlaps(C, (size_t)(r * c * clen) * 8, B, (size_t)(k * c * len2) * 8)) {
        set_error(ctx, "output overlaps an input");
        return PMLG_EALIAS;
    }
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    return poly_mat_mul_device(ctx, C, A, B, r, k, c, len1, len2, p, (cudaStream_t)stream);
}

PMLG_API int pmlg_poly_mat_mulmid(pmlg_ctx *ctx, uint64_t *res, const uint64_t *A, const uint64_t *B,
                                  int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                                  int64_t nlo, int64_t nhi, uint64_t p, int64_t *out_len, void *stream)
{
    PMLG_TRY(check_common(ctx, res, A, B, r, k, c, len1, len2, p));
    if (nlo < 0 || nhi < 0) return PMLG_EINVAL;
    const int64_t cap = nhi > nlo ? nhi - nlo : 0;
    if (overlaps(res, (size_t)(r * c * cap) * 8, A, (size_t)(r * k * len1) * 8) ||
        overlaps(res, (size_t)(r * c * cap) * 8, B, (size_t)(k * c * len2) * 8)) {
        set_error(ctx, "output overlaps an input");
        return PMLG_EALIAS;
    }
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    PMLG_TRY(poly_mat_mulmid_device(ctx, res, A, B, r, k, c, len1, len2, nlo, nhi, p, st));
    if (out_len) {
        // clamp as mulmid.c:505-507 does, with the actual max lengths
        PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, 256));
        unsigned long long *tmp = (unsigned long long *)ctx->ws_aux.ptr;
        int64_t L1 = 0, L2 = 0;
        PMLG_TRY(device_max_length(ctx, A, r * k, len1, len1, tmp, &L1, st));
        PMLG_TRY(device_max_length(ctx, B, k * c, len2, len2, tmp, &L2, st));
        int64_t hi = nhi;
        if (L1 == 0 || L2 == 0) hi = 0;
        else if (hi > L1 + L2 - 1) hi = L1 + L2 - 1;
        *out_len = hi > nlo ? hi - nlo : 0;
    }
    return PMLG_OK;
}

PMLG_API int pmlg_poly_mat_mul_host(pmlg_ctx *ctx, uint64_t *C, const uint64_t *A, const uint64_t *B,
                                    int64_t r, int64_t k, int64_t c, int64_t len1, int64_t len2,
                                    uint64_t p, void *stream)
{
    PMLG_TRY(check_common(ctx, C, A, B, r, k, c, len1, len2, p));
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t clen = (len1 > 0 && len2 > 0) ? len1 + len2 - 1 : 0;
    const size_t bA = (size_t)(r * k * len1) * 8, bB = (size_t)(k * c * len2) * 8,
                 bC = (size_t)(r * c * clen) * 8;
    const size_t oA = 0, oB = (bA + 255) & ~(size_t)255, oC = oB + ((bB + 255) & ~(size_t)255);
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, oC + bC + 256));
    char *base = (char *)ctx->ws_aux.ptr;
    uint64_t *dA = (uint64_t *)(base + oA), *dB = (uint64_t *)(base + oB), *dC = (uint64_t *)(base + oC);
    if (r == 0 || c == 0 || clen == 0 || k == 0) {
        PMLG_TRY(h2d(ctx, dA, A, bA, st));
        PMLG_TRY(h2d(ctx, dB, B, bB, st));
        PMLG_TRY(poly_mat_mul_device(ctx, dC, dA, dB, r, k, c, len1, len2, p, st));
        if (bC) PMLG_CUDA_TRY(cudaMemcpyAsync(C, dC, bC, cudaMemcpyDeviceToHost, st));
        return device_status(ctx, st);
    }
    ProductJob j;
    full_product_job(j, dC, dA, dB, r, k, c, len1, len2, p);
    if (j.lg > kMaxLgN) {
        set_error(ctx, "product length %lld needs a transform beyond 2^%d", (long long)clen, kMaxLgN);
        return PMLG_ELEN;
    }
    CrtPlan plan;
    PMLG_TRY(make_plan(ctx, p, j.lg, k, len1 < len2 ? len1 : len2, &plan));
    PMLG_TRY(ws_reserve(ctx, &ctx->ws, product_scratch_bytes(j, plan)));
    ProductBufs b;
    PMLG_TRY(product_bufs(ctx, j, plan, ctx->ws.ptr, b));
    PMLG_TRY(ensure_side_streams(ctx, 2));
    // The link carries about 210 GB/s to the device and 193 GB/s back, 338 GB/s
    // both ways at once, so the copies in the two directions are made to overlap:
    // B goes first (its transforms follow its chunks), then A in row blocks; each
    // row block of C is transformed, multiplied and transformed back as soon as
    // its rows of A are in, and copied back while the next rows of A arrive.
    cudaStream_t hs = ctx->bstream[0], ds = ctx->bstream[1];
    cudaEvent_t *ev = ctx->hevent;
    const int nb = r >= kHostRowBlocks ? kHostRowBlocks : (int)r;   // row blocks of A and C
    const int64_t nB = k * c;
    const int nbB = nB >= 4 ? 4 : 1;                    // chunks of B
    int ne = 0;
    auto next_event = [&](cudaStream_t s, cudaEvent_t *out) {
        *out = ev[ne++];
        return cudaEventRecord(*out, s) == cudaSuccess ? PMLG_OK : PMLG_ECUDA;
    };
    cudaEvent_t e;
    if (PMLG_HOST_2D && plan.direct && r >= kHostBR && c >= kHostBC && kHostBR * kHostBC > 1) {
        // BR x BC blocks of C.  Block (I, J) needs only rows I of A and columns J of B,
        // so the first block goes back to the host while the rest of the operands are
        // still coming in.  The copies go B columns 0, A rows 0, B columns 1, A rows 1,
        // ...; after B columns s come the blocks (I < s, s), after A rows s the blocks
        // (s, J <= s).  Every block is an ordinary product of its own contiguous device
        // copies (B's column blocks and C's blocks move as 2-D copies, one run of entries
        // per row of entries), and each block of A and of B is transformed once.
        constexpr int BR = kHostBR, BC = kHostBC;
        int64_t R0[BR + 1], C0[BC + 1];
        for (int ib = 0; ib <= BR; ib++) R0[ib] = r * ib / BR;
        for (int jb = 0; jb <= BC; jb++) C0[jb] = c * jb / BC;
        const int64_t N = 1ll << j.lg;
        uint64_t *dBJ[BC];
        for (int jb = 0; jb < BC; jb++) dBJ[jb] = dB + k * C0[jb] * len2;
        uint64_t *dCB[BR][BC];
        {
            uint64_t *w = dC;
            for (int ib = 0; ib < BR; ib++)
                for (int jb = 0; jb < BC; jb++) {
                    dCB[ib][jb] = w;
                    w += (R0[ib + 1] - R0[ib]) * (C0[jb + 1] - C0[jb]) * clen;
                }
        }
        // evaluations: A rows I, B columns J, C blocks (I, J), each in its own point-tiled layout
        uint32_t *EA[BR], *EB[BC], *EC[BR][BC];
        PMLG_TRY(ws_reserve(ctx, &ctx->ws, product_scratch_bytes(j, plan) + (BR + BC + BR * BC) * 256));
        {
            char *w = (char *)ctx->ws.ptr;
            auto take = [&](int64_t nent) {
                uint32_t *r_ = (uint32_t *)w;
                w += align256((size_t)(N * nent) * 4);
                return r_;
            };
            for (int ib = 0; ib < BR; ib++) EA[ib] = take((R0[ib + 1] - R0[ib]) * k);
            for (int jb = 0; jb < BC; jb++) EB[jb] = take(k * (C0[jb + 1] - C0[jb]));
            for (int ib = 0; ib < BR; ib++)
                for (int jb = 0; jb < BC; jb++) EC[ib][jb] = take((R0[ib + 1] - R0[ib]) * (C0[jb + 1] - C0[jb]));
        }
        // the product of block (I, J) and its buffers
        auto block_job = [&](int ib, int jb, ProductJob &bj, ProductBufs &bb) {
            bj = j;
            bj.r = R0[ib + 1] - R0[ib];
            bj.c = C0[jb + 1] - C0[jb];
            bj.A = dA + R0[ib] * k * len1;
            bj.B = dBJ[jb];
            bj.C = dCB[ib][jb];
            bb = b;
            bb.EA = EA[ib];
            bb.EB = EB[jb];
            bb.EC = EC[ib][jb];
            bb.R32 = nullptr;
        };
        PMLG_TRY(next_event(st, &e));
        PMLG_CUDA_TRY(cudaStreamWaitEvent(hs, e, 0));
        PMLG_CUDA_TRY(cudaStreamWaitEvent(ds, e, 0));
        cudaEvent_t bev[BC], aev[BR];
        const int nsteps = BR > BC ? BR : BC;
        for (int q = 0; q < nsteps; q++) {   // B columns q, A rows q
            if (q < BC) {
                const int64_t bw = C0[q + 1] - C0[q];
                PMLG_CUDA_TRY(cudaMemcpy2DAsync(dBJ[q], (size_t)(bw * len2) * 8, B + C0[q] * len2,
                                                (size_t)(c * len2) * 8, (size_t)(bw * len2) * 8, (size_t)k,
                                                cudaMemcpyHostToDevice, hs));
                PMLG_TRY(next_event(hs, &bev[q]));
            }
            if (q < BR) {
                PMLG_TRY(h2d(ctx, dA + R0[q] * k * len1, A + R0[q] * k * len1,
                             (size_t)((R0[q + 1] - R0[q]) * k * len1) * 8, hs));
                PMLG_TRY(next_event(hs, &aev[q]));
            }
        }
        auto run_block = [&](int ib, int jb) -> int {
            ProductJob bj;
            ProductBufs bb;
            block_job(ib, jb, bj, bb);
            PMLG_TRY(product_pointwise(ctx, bj, plan, bb, 0, bj.r, ctx->form, st));
            PMLG_TRY(product_inverse(ctx, bj, plan, bb, 0, bj.r * bj.c, st));
            cudaEvent_t ce;
            PMLG_TRY(next_event(st, &ce));
            PMLG_CUDA_TRY(cudaStreamWaitEvent(ds, ce, 0));
            PMLG_CUDA_TRY(cudaMemcpy2DAsync(C + (R0[ib] * c + C0[jb]) * clen, (size_t)(c * clen) * 8, bj.C,
                                            (size_t)(bj.c * clen) * 8, (size_t)(bj.c * clen) * 8, (size_t)bj.r,
                                            cudaMemcpyDeviceToHost, ds));
            return PMLG_OK;
        };
        auto fwd_block = [&](int which, int h) -> int {   // A rows h (which 0) or B columns h (which 1)
            ProductJob bj;
            ProductBufs bb;
            block_job(which == 0 ? h : 0, which == 0 ? 0 : h, bj, bb);
            return product_forward(ctx, bj, plan, bb, which, 0, which == 0 ? bj.r * k : k * bj.c, st);
        };
        for (int q = 0; q < nsteps; q++) {
            if (q < BC) {
                PMLG_CUDA_TRY(cudaStreamWaitEvent(st, bev[q], 0));
                PMLG_TRY(fwd_block(1, q));
                for (int ib = 0; ib < q && ib < BR; ib++) PMLG_TRY(run_block(ib, q));
            }
            if (q < BR) {
                PMLG_CUDA_TRY(cudaStreamWaitEvent(st, aev[q], 0));
                PMLG_TRY(fwd_block(0, q));
                for (int jb = 0; jb <= q && jb < BC; jb++) PMLG_TRY(run_block(q, jb));
            }
        }
        PMLG_TRY(next_event(ds, &e));
        PMLG_CUDA_TRY(cudaStreamWaitEvent(st, e, 0));
        return device_status(ctx, st);
    }
    PMLG_TRY(next_event(st, &e));
    PMLG_CUDA_TRY(cudaStreamWaitEvent(hs, e, 0));
    PMLG_CUDA_TRY(cudaStreamWaitEvent(ds, e, 0));
    for (int q = 0; q < nbB; q++) {
        const int64_t f0 = nB * q / nbB, f1 = nB * (q + 1) / nbB;
        PMLG_TRY(h2d(ctx, dB + f0 * len2, B + f0 * len2, (size_t)((f1 - f0) * len2) * 8, hs));
        PMLG_TRY(next_event(hs, &e));
        PMLG_CUDA_TRY(cudaStreamWaitEvent(st, e, 0));
        PMLG_TRY(product_forward(ctx, j, plan, b, 1, f0, f1, st));
    }
    cudaEvent_t arows[kHostRowBlocks];
    for (int i = 0; i < nb; i++) {
        const int64_t i0 = r * i / nb, i1 = r * (i + 1) / nb;
        PMLG_TRY(h2d(ctx, dA + i0 * k * len1, A + i0 * k * len1, (size_t)((i1 - i0) * k * len1) * 8, hs));
        PMLG_TRY(next_event(hs, &arows[i]));
    }
    for (int i = 0; i < nb; i++) {
        const int64_t i0 = r * i / nb, i1 = r * (i + 1) / nb;
        PMLG_CUDA_TRY(cudaStreamWaitEvent(st, arows[i], 0));
        PMLG_TRY(product_forward(ctx, j, plan, b, 0, i0 * k, i1 * k, st));
        PMLG_TRY(product_pointwise(ctx, j, plan, b, i0, i1, ctx->form, st));
        PMLG_TRY(product_inverse(ctx, j, plan, b, i0 * c, i1 * c, st));
        PMLG_TRY(next_event(st, &e));
        PMLG_CUDA_TRY(cudaStreamWaitEvent(ds, e, 0));
        PMLG_CUDA_TRY(cudaMemcpyAsync(C + i0 * c * clen, dC + i0 * c * clen, (size_t)((i1 - i0) * c * clen) * 8,
                                      cudaMemcpyDeviceToHost, ds));
    }
    PMLG_TRY(next_event(ds, &e));
    PMLG_CUDA_TRY(cudaStreamWaitEvent(st, e, 0));
    return device_status(ctx, st);
}

PMLG_API int pmlg_poly_mat_mulmid_host(pmlg_ctx *ctx, uint64_t *res, const uint64_t *A,
                                       const uint64_t *B, int64_t r, int64_t k, int64_t c,
                                       int64_t len1, int64_t len2, int64_t nlo, int64_t nhi,
                                       uint64_t p, int64_t *out_len, void *stream)
{
    PMLG_TRY(check_common(ctx, res, A, B, r, k, c, len1, len2, p));
    if (nlo < 0 || nhi < 0) return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t cap = nhi > nlo ? nhi - nlo : 0;
    const size_t bA = (size_t)(r * k * len1) * 8, bB = (size_t)(k * c * len2) * 8,
                 bC = (size_t)(r * c * cap) * 8;
    const size_t oA = 0, oB = (bA + 255) & ~(size_t)255, oC = oB + ((bB + 255) & ~(size_t)255);
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, oC + bC + 512));
    char *base = (char *)ctx->ws_aux.ptr;
    uint64_t *dA = (uint64_t *)(base + oA), *dB = (uint64_t *)(base + oB), *dC = (uint64_t *)(base + oC);
    PMLG_TRY(h2d(ctx, dA, A, bA, st));
    PMLG_TRY(h2d(ctx, dB, B, bB, st));
    PMLG_TRY(poly_mat_mulmid_device(ctx, dC, dA, dB, r, k, c, len1, len2, nlo, nhi, p, st));
    if (bC) PMLG_CUDA_TRY(cudaMemcpyAsync(res, dC, bC, cudaMemcpyDeviceToHost, st));
    PMLG_TRY(device_status(ctx, st));
    if (out_len) {
        // the actual max lengths are read on the host copies
        auto hostlen = [](const uint64_t *P, int64_t nent, int64_t len) {
            int64_t L = 0;
            for (int64_t e = 0; e < nent; e++)
                for (int64_t d = len - 1; d >= L; d--)
                    if (P[e * len + d]) { L = d + 1; break; }
            return L;
        };
        const int64_t L1 = hostlen(A, r * k, len1), L2 = hostlen(B, k * c, len2);
        int64_t hi = nhi;
        if (L1 == 0 || L2 == 0) hi = 0;
        else if (hi > L1 + L2 - 1) hi = L1 + L2 - 1;
        *out_len = hi > nlo ? hi - nlo : 0;
    }
    return PMLG_OK;
}

PMLG_API int pmlg_poly_mat_mul_batch(pmlg_ctx *ctx, const pmlg_polymat_job *jobs, int64_t njobs,
                                     void *stream)
{
    if (!ctx || (njobs > 0 && !jobs) || njobs < 0) return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    // 1. validate every job, build its transform plan and tables (host work, before any launch)
    struct Item
    {
        ProductJob j;
        CrtPlan plan;
        size_t scratch;
        double work;
    };
    std::vector<Item> items;
    items.reserve((size_t)njobs);
    for (int64_t i = 0; i < njobs; i++) {
        const pmlg_polymat_job &J = jobs[i];
        PMLG_TRY(check_common(ctx, J.C, J.A, J.B, J.r, J.k, J.c, J.len1, J.len2, J.p));
        const int64_t clen = (J.len1 > 0 && J.len2 > 0) ? J.len1 + J.len2 - 1 : 0;
        if (J.r == 0 || J.c == 0 || clen == 0) continue;
        if (J.k == 0) {
            PMLG_CUDA_TRY(cudaMemsetAsync(J.C, 0, (size_t)(J.r * J.c * clen) * 8, st));
            continue;
        }
        Item it{};
        ProductJob &j = it.j;
        full_product_job(j, J.C, J.A, J.B, J.r, J.k, J.c, J.len1, J.len2, J.p);
        if (j.lg > kMaxLgN) {
            set_error(ctx, "job %lld: product length %lld needs a transform beyond 2^%d", (long long)i,
                      (long long)clen, kMaxLgN);
            return PMLG_ELEN;
        }
        const int64_t minlen = j.a_len < j.b_len ? j.a_len : j.b_len;
        PMLG_TRY(make_plan(ctx, j.p, j.lg, j.k, minlen, &it.plan));
        for (int q = 0; q < it.plan.t; q++) {
            const NttTable *tab;
            PMLG_TRY(get_table(ctx, it.plan.q[q], j.lg, &tab));
        }
        it.scratch = (product_scratch_bytes(j, it.plan) + 255) & ~(size_t)255;
        const double N = (double)(1ll << j.lg);
        it.work = it.plan.t * N * ((double)(j.r * j.k + j.k * j.c + j.r * j.c) * j.lg + (double)j.r * j.k * j.c);
        items.push_back(it);
    }
    if (items.empty()) return PMLG_OK;
    // 2. spread the jobs over the batch streams, largest first onto the least loaded stream;
    //    each stream owns a scratch region as large as its largest job
    const int K = (int)(items.size() < (size_t)pmlg_ctx::kBatchStreams ? items.size() : pmlg_ctx::kBatchStreams);
    std::vector<int> order(items.size());
    for (size_t i = 0; i < items.size(); i++) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return items[a].work > items[b].work; });
    std::vector<int> slot(items.size());
    std::vector<double> load(K, 0.0);
    std::vector<size_t> need(K, 0);
    for (int idx : order) {
        int s = 0;
        for (int t = 1; t < K; t++)
            if (load[t] < load[s]) s = t;
        slot[idx] = s;
        load[s] += items[idx].work;
        if (items[idx].scratch > need[s]) need[s] = items[idx].scratch;
    }
    std::vector<size_t> off(K, 0);
    size_t total = 0;
    for (int s = 0; s < K; s++) {
        off[s] = total;
        total += need[s];
    }
    PMLG_TRY(ws_reserve(ctx, &ctx->ws_batch, total));
    PMLG_TRY(ensure_side_streams(ctx, K));
    // 3. fork from the caller's stream, run, join back
    char *base = (char *)ctx->ws_batch.ptr;
    auto launch_all = [&]() -> int {
        PMLG_CUDA_TRY(cudaEventRecord(ctx->bevent[K], st));
        for (int s = 0; s < K; s++) PMLG_CUDA_TRY(cudaStreamWaitEvent(ctx->bstream[s], ctx->bevent[K], 0));
        for (int idx : order) {
            const int s = slot[idx];
            PMLG_TRY(product_run(ctx, items[idx].j, items[idx].plan, base + off[s], ctx->form, ctx->bstream[s]));
        }
        for (int s = 0; s < K; s++) {
            PMLG_CUDA_TRY(cudaEventRecord(ctx->bevent[s], ctx->bstream[s]));
            PMLG_CUDA_TRY(cudaStreamWaitEvent(st, ctx->bevent[s], 0));
        }
        return PMLG_OK;
    };
    // A batch seen again (same jobs, pointers, moduli, form and scratch) is captured
    // into a CUDA graph on its second call and replayed from then on: one launch of the
    // whole fork / products / join instead of one per kernel.  The first call of a batch
    // launches directly (it also builds every table and tunes every form the batch needs,
    // host work that a capture must not contain).
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PMLG_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
    if (!ctx->batch_graphs || ctx->profiling || cs != cudaStreamCaptureStatusNone) return launch_all();
    // the batch's full description (every pointer, shape and modulus, the form, the
    // scratch and the stream) and its hash; a stored graph is replayed only when the
    // whole description matches, not the hash alone
    uint64_t key = 1469598103934665603ull;
    std::vector<uint64_t> sig;
    sig.reserve(5 + 9 * (size_t)njobs);
    auto mix = [&](uint64_t v) {
        sig.push_back(v);
        for (int b = 0; b < 8; b++) {
            key ^= (v >> (8 * b)) & 0xff;
            key *= 1099511628211ull;
        }
    };
    mix((uint64_t)njobs); mix((uint64_t)ctx->form); mix((uint64_t)(uintptr_t)base); mix((uint64_t)total);
    mix((uint64_t)(uintptr_t)st);
    for (int64_t i = 0; i < njobs; i++) {
        const pmlg_polymat_job &J = jobs[i];
        mix((uint64_t)(uintptr_t)J.C); mix((uint64_t)(uintptr_t)J.A); mix((uint64_t)(uintptr_t)J.B);
        mix((uint64_t)J.r); mix((uint64_t)J.k); mix((uint64_t)J.c); mix((uint64_t)J.len1); mix((uint64_t)J.len2);
        mix(J.p);
    }
    for (auto &g : ctx->bgraph)
        if (g.exec && g.key == key && g.sig == sig) {
            PMLG_CUDA_TRY(cudaGraphLaunch(g.exec, st));
            count_launch(ctx, (unsigned)g.launches);
            return PMLG_OK;
        }
    if (ctx->batch_seen != key || ctx->batch_seen_sig != sig) {
        ctx->batch_seen = key;
        ctx->batch_seen_sig = sig;
        return launch_all();
    }
    // second call of this batch: capture, instantiate, launch
    const unsigned long long l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    int s = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess ? PMLG_OK : PMLG_ECUDA;
    if (s == PMLG_OK) {
        s = launch_all();
        if (cudaStreamEndCapture(st, &graph) != cudaSuccess && s == PMLG_OK) s = PMLG_ECUDA;
    }
    cudaGraphExec_t exec = nullptr;
    if (s == PMLG_OK && graph && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) s = PMLG_ECUDA;
    if (graph) cudaGraphDestroy(graph);
    const unsigned long long recorded = ctx->launches - l0;   // kernels the capture recorded
    ctx->launches = l0;
    if (s != PMLG_OK || !exec) {
        // the capture failed: clear its error, launch directly, and leave graphs off for
        // this context (pmlg_ctx_set_batch_graphs turns them back on)
        (void)cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        ctx->batch_graphs = 0;
        return launch_all();
    }
    pmlg_ctx::BatchGraph &slotg = ctx->bgraph[ctx->bgraph_next];
    ctx->bgraph_next = (ctx->bgraph_next + 1) % pmlg_ctx::kBatchGraphs;
    if (slotg.exec) cudaGraphExecDestroy(slotg.exec);
    slotg.exec = exec;
    slotg.key = key;
    slotg.sig = std::move(sig);
    slotg.launches = recorded;
    PMLG_CUDA_TRY(cudaGraphLaunch(exec, st));
    count_launch(ctx, (unsigned)slotg.launches);
    return PMLG_OK;
}

}  // extern "C"
