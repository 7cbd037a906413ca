// context.cu -- context, scratch memory, NTT tables and CRT plans.
#include "pmlg_internal.cuh"
#include "pointwise.cuh"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

namespace pmlg {

void set_error(pmlg_ctx *ctx, const char *fmt, ...)
{
    if (!ctx)
        return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->last_error, sizeof(ctx->last_error), fmt, ap);
    va_end(ap);
}

typedef unsigned __int128 u128;

uint64_t h_mulmod(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)(((u128)a * b) % p); }

uint64_t h_powmod(uint64_t a, uint64_t e, uint64_t p)
{
    uint64_t r = 1 % p;
    a %= p;
    while (e) {
        if (e & 1) r = h_mulmod(r, a, p);
        a = h_mulmod(a, a, p);
        e >>= 1;
    }
    return r;
}

uint64_t h_invmod(uint64_t a, uint64_t p)
{
    __int128 t = 0, nt = 1, r = p, nr = a % p;
    while (nr != 0) {
        __int128 qq = r / nr, tmp;
        tmp = t - qq * nt; t = nt; nt = tmp;
        tmp = r - qq * nr; r = nr; nr = tmp;
    }
    if (r != 1) return 0;
    if (t < 0) t += p;
    return (uint64_t)t;
}

bool h_is_prime(uint64_t n)
{
    if (n < 2) return false;
    static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (uint64_t s : small) {
        if (n == s) return true;
        if (n % s == 0) return false;
    }
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) { d >>= 1; s++; }
    for (uint64_t a : small) {
        uint64_t x = h_powmod(a, d, n);
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int r = 1; r < s; r++) {
            x = h_mulmod(x, x, n);
            if (x == n - 1) { comp = false; break; }
        }
        if (comp) return false;
    }
    return true;
}

// generator of (Z/qZ)^*, q prime
static uint64_t primitive_root(uint64_t q)
{
    uint64_t pm1 = q - 1, fac[64];
    int nf = 0;
    uint64_t t = pm1;
    for (uint64_t f = 2; f * f <= t; f++)
        if (t % f == 0) { fac[nf++] = f; while (t % f == 0) t /= f; }
    if (t > 1) fac[nf++] = t;
    for (uint64_t g = 2;; g++) {
        bool ok = true;
        for (int i = 0; i < nf; i++)
            if (h_powmod(g, pm1 / fac[i], q) == 1) { ok = false; break; }
        if (ok) return g;
    }
}

int get_table(pmlg_ctx *ctx, uint32_t q, int lg, const NttTable **out)
{
    for (int i = 0; i < ctx->ntables; i++)
        if (ctx->tables[i].q == q && ctx->tables[i].lg == lg) {
            *out = &ctx->tables[i];
            return PMLG_OK;
        }
    if (ctx->ntables >= pmlg_ctx::kMaxTables) {
        set_error(ctx, "NTT table cache full");
        return PMLG_ENOMEM;
    }
    const uint64_t N = 1ull << lg;
    if (q >= (1u << 30) || ((uint64_t)q - 1) % N != 0) {
        set_error(ctx, "q=%u has no root of unity of order 2^%d", q, lg);
        return PMLG_ENOROOT;
    }
    const uint64_t g = primitive_root(q);
    const uint64_t wN = h_powmod(g, (q - 1) / N, q);
    const uint64_t iwN = h_invmod(wN, q);
    uint32_t *hw = (uint32_t *)malloc(4 * N * sizeof(uint32_t));
    if (!hw) return PMLG_ENOMEM;
    // interleaved {w^e, quotient} pairs: forward powers in [0, 2N), inverse in [2N, 4N)
    uint32_t *hf = hw, *hi = hw + 2 * N;
    {
        uint64_t x = 1, y = 1;
        for (uint64_t j = 0; j < N; j++) {
            hf[2 * j] = (uint32_t)x; hf[2 * j + 1] = h_shoup_q((uint32_t)x, q);
            hi[2 * j] = (uint32_t)y; hi[2 * j + 1] = h_shoup_q((uint32_t)y, q);
            x = h_mulmod(x, wN, q);
            y = h_mulmod(y, iwN, q);
        }
    }
    // consistency: w^N = 1 and w^(N/2) = -1, so w is a primitive N-th root
    if (h_mulmod(hf[2 * (N - 1)], wN, q) != 1 || hf[2 * (N / 2)] != q - 1) {
        free(hw);
        set_error(ctx, "root of unity check failed");
        return PMLG_EINVAL;
    }
    // exact check of every Shoup quotient: w' * q <= w * 2^32 < (w' + 1) * q
    for (uint64_t i = 0; i < 2 * N; i++) {
        const uint32_t w = hw[2 * i], wq = hw[2 * i + 1];
        const u128 lhs = (u128)wq * q, rhs = (u128)w << 32;
        if (!(w < q && lhs <= rhs && rhs < lhs + q)) {
            free(hw);
            set_error(ctx, "Shoup quotient check failed");
            return PMLG_EINVAL;
        }
    }
    // group twiddle tables (layout in pmlg_internal.cuh), copied out of the power tables
    const uint64_t G = 15 * (N >> 3);   // >= 15 * (2^(lg-3) - 1) entries per direction
    uint32_t *hg = (uint32_t *)calloc(4 * G, sizeof(uint32_t));
    if (!hg) { free(hw); return PMLG_ENOMEM; }
    for (int lls = 0; lls <= lg - 4; lls++) {
        const uint64_t L = 1ull << lls, base = 15 * (L - 1);
        for (uint64_t m = 1; m < 16; m++) {
            const uint64_t br = ((m & 1) << 3) | ((m & 2) << 1) | ((m & 4) >> 1) | ((m & 8) >> 3);
            for (uint64_t off = 0; off < L; off++) {
                const uint64_t ex = (off * br) << (lg - lls - 4);   // < N
                const uint64_t i = base + (m - 1) * L + off;
                hg[2 * i] = hf[2 * ex]; hg[2 * i + 1] = hf[2 * ex + 1];
                hg[2 * G + 2 * i] = hi[2 * ex]; hg[2 * G + 2 * i + 1] = hi[2 * ex + 1];
            }
        }
    }
    free(hw);
    NttTable T;
    T.q = q;
    T.lg = lg;
    void *d = nullptr;
    cudaError_t e = cudaMalloc(&d, 4 * G * sizeof(uint32_t));
    if (e != cudaSuccess) {
        free(hg);
        set_error(ctx, "cudaMalloc tables: %s", cudaGetErrorString(e));
        return PMLG_ENOMEM;
    }
    e = cudaMemcpy(d, hg, 4 * G * sizeof(uint32_t), cudaMemcpyHostToDevice);
    free(hg);
    if (e != cudaSuccess) {
        cudaFree(d);
        set_error(ctx, "cudaMemcpy tables: %s", cudaGetErrorString(e));
        return PMLG_ECUDA;
    }
    T.d_w = (uint2 *)d;
    T.d_iw = T.d_w + G;
    for (int j = 0; j < 8; j++) {
        const uint64_t ex = (uint64_t)j * (N / 16);
        T.c16[j] = (uint32_t)h_powmod(wN, ex, q);
        T.c16q[j] = h_shoup_q(T.c16[j], q);
        T.ic16[j] = (uint32_t)h_powmod(iwN, ex, q);
        T.ic16q[j] = h_shoup_q(T.ic16[j], q);
    }
    T.ninv = (uint32_t)h_invmod(N % q, q);
    T.ninvq = h_shoup_q(T.ninv, q);
    T.r32 = (uint32_t)((1ull << 32) % q);
    T.r32q = h_shoup_q(T.r32, q);
    T.oneq = (uint32_t)((1ull << 32) / q);
    ctx->tables[ctx->ntables] = T;
    *out = &ctx->tables[ctx->ntables];
    ctx->ntables++;
    return PMLG_OK;
}

// 30-bit primes q = c * 2^e + 1 with e >= 21, largest first
static const uint32_t kCrtPrimes[] = {1012924417u, 1004535809u, 998244353u, 985661441u,
                                      975175681u, 962592769u, 950009857u, 943718401u};

int make_plan(pmlg_ctx *ctx, uint64_t p, int lg, int64_t inner, int64_t minlen, CrtPlan *plan)
{
    memset(plan, 0, sizeof(*plan));
    plan->p = p;
    if (p < 2) {
        set_error(ctx, "modulus %llu < 2", (unsigned long long)p);
        return PMLG_EBADMOD;
    }
    if (p < (1ull << 30) && ((p - 1) >> lg) << lg == p - 1 && h_is_prime(p)) {
        plan->direct = 1;
        plan->t = 1;
        plan->q[0] = (uint32_t)p;
        plan->qp[0] = 0;
        return PMLG_OK;
    }
    if (lg > 21) {
        set_error(ctx, "transform length 2^%d too large for the CRT primes", lg);
        return PMLG_ELEN;
    }
    // bits of the bound inner * minlen * (p-1)^2 (strictly below 2^bits)
    u128 pm1 = p - 1;
    double bits = 0;
    {
        // exact enough: compute log2 of each factor with integer bit lengths + 1
        auto blen = [](u128 x) { int b = 0; while (x) { b++; x >>= 1; } return b; };
        bits = 2.0 * blen(pm1) + blen((u128)(inner > 0 ? inner : 1)) + blen((u128)(minlen > 0 ? minlen : 1));
    }
    // each prime contributes more than 29.8 bits; require strictly more bits than the bound
    int t = 0;
    double have = 0;
    const int navail = (int)(sizeof(kCrtPrimes) / sizeof(kCrtPrimes[0]));
    while (have <= bits && t < navail) {
        // log2(q) >= 29.8 for all listed primes
        have += 29.8;
        t++;
    }
    if (have <= bits || t > kMaxPrimes) {
        set_error(ctx, "modulus too large for %d CRT primes", kMaxPrimes);
        return PMLG_EBADMOD;
    }
    plan->direct = 0;
    plan->t = t;
    for (int j = 0; j < t; j++) plan->q[j] = kCrtPrimes[j];
    for (int j = 0; j < t; j++) {
        const uint32_t qj = plan->q[j];
        uint64_t pr = 1;
        for (int l = 0; l < j; l++) {
            plan->qmod[j][l] = plan->q[l] % qj;
            plan->qmodq[j][l] = h_shoup_q(plan->qmod[j][l], qj);
            pr = h_mulmod(pr, plan->q[l] % qj, qj);
        }
        plan->ginv[j] = (j == 0) ? 1 : (uint32_t)h_invmod(pr, qj);
        plan->ginvq[j] = h_shoup_q(plan->ginv[j], qj);
        plan->qp[j] = plan->q[j] % p;
        plan->qpq[j] = (uint64_t)(((unsigned __int128)plan->qp[j] << 64) / p);
    }
    plan->onepq = (uint64_t)(((unsigned __int128)1 << 64) / p);
    return PMLG_OK;
}

int ws_reserve(pmlg_ctx *ctx, Workspace *ws, size_t bytes)
{
    if (ws->bytes >= bytes)
        return PMLG_OK;
    if (ws->ptr) {
        // the old buffer may still be in use by queued work on any stream
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            set_error(ctx, "sync before scratch growth: %s", cudaGetErrorString(e));
            return PMLG_ECUDA;
        }
        cudaFree(ws->ptr);
        ws->ptr = nullptr;
        ws->bytes = 0;
    }
    size_t sz = bytes + (bytes >> 3) + 256;
    cudaError_t e = cudaMalloc(&ws->ptr, sz);
    if (e != cudaSuccess) {
        ws->ptr = nullptr;
        set_error(ctx, "cudaMalloc scratch (%zu bytes): %s", sz, cudaGetErrorString(e));
        return PMLG_ENOMEM;
    }
    ws->bytes = sz;
    return PMLG_OK;
}

static cudaEvent_t pool_event(pmlg_ctx *ctx)
{
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_begin(pmlg_ctx *ctx, const char *name, cudaStream_t st)
{
    if (!ctx->profiling) return;
    ProfRecord r{name, pool_event(ctx), pool_event(ctx)};
    cudaEventRecord(r.beg, st);
    ctx->prof.push_back(r);
}

void prof_end(pmlg_ctx *ctx, cudaStream_t st)
{
    if (!ctx->profiling || ctx->prof.empty()) return;
    cudaEventRecord(ctx->prof.back().end, st);
}

int device_status(pmlg_ctx *ctx, cudaStream_t st)
{
    int h = 0;
    PMLG_CUDA_TRY(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    if (h) {
        PMLG_CUDA_TRY(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), st));
        PMLG_CUDA_TRY(cudaStreamSynchronize(st));
        set_error(ctx, "a bounded device wait gave up: the results of the calls since the last check are invalid");
        return PMLG_ETIMEOUT;
    }
    return PMLG_OK;
}

// Waits on an mbarrier phase that nothing completes, for at most wait_ns, and
// records the give-up in the error word exactly as the production kernels do:
// the path by which a stuck wait reaches the host, exercised without a fault.
__global__ void selftest_wait_kernel(int *err, unsigned long long wait_ns)
{
    __shared__ __align__(8) unsigned long long bar;
    const unsigned addr = (unsigned)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(addr));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    __syncthreads();
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    unsigned done = 0;
    for (int it = 0; it < (1 << 26) && !done; it++) {
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(addr) : "memory");
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > wait_ns) break;
    }
    if (!done && threadIdx.x == 0) atomicExch(err, 1);
}

}  // namespace pmlg

using namespace pmlg;

extern "C" {

PMLG_API int pmlg_ctx_create(pmlg_ctx **out, int device)
{
    if (!out) return PMLG_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PMLG_ECUDA;
    if (device < 0 || device >= ndev) return PMLG_EINVAL;
    pmlg_ctx *ctx = new (std::nothrow) pmlg_ctx();
    if (!ctx) return PMLG_ENOMEM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return PMLG_ECUDA; }
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess || cudaMemset(ctx->d_err, 0, sizeof(int)) != cudaSuccess) {
        delete ctx;
        return PMLG_ENOMEM;
    }
    *out = ctx;
    return PMLG_OK;
}

PMLG_API int pmlg_ctx_destroy(pmlg_ctx *ctx)
{
    if (!ctx) return PMLG_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (int i = 0; i < ctx->ntables; i++) cudaFree(ctx->tables[i].d_w);
    if (ctx->ws.ptr) cudaFree(ctx->ws.ptr);
    if (ctx->ws_aux.ptr) cudaFree(ctx->ws_aux.ptr);
    if (ctx->ws_pm.ptr) cudaFree(ctx->ws_pm.ptr);
    if (ctx->ws_batch.ptr) cudaFree(ctx->ws_batch.ptr);
    for (int i = 0; i < pmlg_ctx::kBatchStreams; i++)
        if (ctx->bstream[i]) cudaStreamDestroy(ctx->bstream[i]);
    for (int i = 0; i <= pmlg_ctx::kBatchStreams; i++)
        if (ctx->bevent[i]) cudaEventDestroy(ctx->bevent[i]);
    for (int i = 0; i < pmlg_ctx::kHostEvents; i++)
        if (ctx->hevent[i]) cudaEventDestroy(ctx->hevent[i]);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    for (auto &r : ctx->prof) { cudaEventDestroy(r.beg); cudaEventDestroy(r.end); }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    for (auto &g : ctx->bgraph)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    delete ctx;
    return PMLG_OK;
}

PMLG_API int pmlg_ctx_set_form(pmlg_ctx *ctx, int form)
{
    if (!ctx || form < PMLG_FORM_AUTO || form > PMLG_FORM_F16_TC) return PMLG_EINVAL;
    ctx->form = form;
    return PMLG_OK;
}

PMLG_API int pmlg_ctx_set_tuning(pmlg_ctx *ctx, int on)
{
    if (!ctx) return PMLG_EINVAL;
    ctx->tuning = on ? 1 : 0;
    return PMLG_OK;
}

PMLG_API int pmlg_ctx_tuned_form(const pmlg_ctx *ctx, int r, int k, int c, int64_t npts)
{
    if (!ctx || r < 1 || r > 64 || k < 1 || k > 64 || c < 1 || c > 64 || npts < 1) return -PMLG_EINVAL;
    auto it = ctx->tuned.find(tune_key(r, k, c, npts));
    return it == ctx->tuned.end() ? PMLG_FORM_AUTO : it->second;
}

PMLG_API int pmlg_ctx_set_batch_graphs(pmlg_ctx *ctx, int on)
{
    if (!ctx) return PMLG_EINVAL;
    ctx->batch_graphs = on ? 1 : 0;
    if (!on) ctx->batch_seen = 0;
    return PMLG_OK;
}

PMLG_API int pmlg_ctx_set_leaf_order(pmlg_ctx *ctx, int64_t order)
{
    if (!ctx || order < 0) return PMLG_EINVAL;
    ctx->leaf_order = order;
    return PMLG_OK;
}

PMLG_API unsigned long long pmlg_ctx_launch_count(const pmlg_ctx *ctx)
{
    return ctx ? ctx->launches : 0ull;
}

PMLG_API int pmlg_ctx_set_profiling(pmlg_ctx *ctx, int on)
{
    if (!ctx) return PMLG_EINVAL;
    cudaSetDevice(ctx->device);
    for (auto &r : ctx->prof) {
        ctx->event_pool.push_back(r.beg);
        ctx->event_pool.push_back(r.end);
    }
    ctx->prof.clear();
    ctx->profiling = on ? 1 : 0;
    return PMLG_OK;
}

PMLG_API int pmlg_ctx_profile_read(pmlg_ctx *ctx, char *names, size_t names_len, double *ms,
                                   unsigned long long *counts, int max_kernels, int *n_out)
{
    if (!ctx || !n_out || (max_kernels > 0 && (!ms || !counts))) return PMLG_EINVAL;
    cudaSetDevice(ctx->device);
    std::vector<const char *> keys;
    std::vector<double> tot;
    std::vector<unsigned long long> cnt;
    for (auto &r : ctx->prof) {
        if (cudaEventSynchronize(r.end) != cudaSuccess) return PMLG_ECUDA;
        float t = 0.f;
        if (cudaEventElapsedTime(&t, r.beg, r.end) != cudaSuccess) return PMLG_ECUDA;
        size_t i = 0;
        while (i < keys.size() && strcmp(keys[i], r.name) != 0) i++;
        if (i == keys.size()) { keys.push_back(r.name); tot.push_back(0); cnt.push_back(0); }
        tot[i] += t;
        cnt[i] += 1;
    }
    const int n = (int)keys.size() < max_kernels ? (int)keys.size() : max_kernels;
    size_t pos = 0;
    if (names && names_len) names[0] = 0;
    for (int i = 0; i < n; i++) {
        ms[i] = tot[i];
        counts[i] = cnt[i];
        if (names) {
            const size_t l = strlen(keys[i]);
            if (pos + l + 2 <= names_len) {
                memcpy(names + pos, keys[i], l);
                pos += l;
                names[pos++] = '\n';
                names[pos] = 0;
            }
        }
    }
    *n_out = n;
    return PMLG_OK;
}

PMLG_API const char *pmlg_ctx_last_error(const pmlg_ctx *ctx)
{
    return ctx ? ctx->last_error : "null context";
}

PMLG_API int pmlg_ctx_device_status(pmlg_ctx *ctx, void *stream)
{
    if (!ctx) return PMLG_EINVAL;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    return pmlg::device_status(ctx, (cudaStream_t)stream);
}

PMLG_API int pmlg_ctx_selftest_timeout(pmlg_ctx *ctx, unsigned long long wait_ns, void *stream)
{
    if (!ctx || wait_ns == 0 || wait_ns > 1000000000ull) return PMLG_EINVAL;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    pmlg::selftest_wait_kernel<<<1, 32, 0, st>>>(ctx->d_err, wait_ns);
    pmlg::count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return pmlg::device_status(ctx, st);
}

PMLG_API const char *pmlg_strerror(int status)
{
    switch (status) {
    case PMLG_OK: return "ok";
    case PMLG_EINVAL: return "invalid argument";
    case PMLG_EBADMOD: return "unsupported modulus";
    case PMLG_ENOROOT: return "no root of unity of the needed order";
    case PMLG_ELEN: return "length beyond the supported transform size";
    case PMLG_EALIAS: return "output overlaps an input";
    case PMLG_ETIMEOUT: return "bounded device wait gave up";
    case PMLG_ECUDA: return "CUDA runtime error";
    case PMLG_ENOMEM: return "allocation failed";
    case PMLG_EUNSUP: return "unsupported shape";
    default: return "unknown status";
    }
}

}  // extern "C"
