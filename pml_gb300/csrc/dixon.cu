// dixon.cu -- truncated inverse and x-adic Dixon lifting of polynomial matrices:
// nmod_poly_mat_inv_trunc and nmod_poly_mat_dixon
// (flint-extras/src/nmod_poly_mat_extra/nmod_poly_mat_dixon.c:32-143).
//
// The inverse mod x^order comes from the approximant basis of [A \\ -I] at order with
// shift [0, ..., 0, order, ..., order] (the device pmbasis); A(0) is invertible
// exactly when the basis' bottom-right block is the identity, and the inverse is its
// bottom-left block.  Dixon lifting then produces one x-adic digit of X per step with
// the library's middle product and product, and one fused kernel forms the next
// residue (B - A S) div x^order.  The two left operands that every step shares, the
// truncated inverse and A, are transformed once: their evaluations are kept across
// the steps, as _nmod_poly_mat_mul_geometric_precomp keeps them
// (mul_geometric.c:32-119).  Every matrix stays in device memory.
#include "pmlg_internal.cuh"
#include "ntt.cuh"
#include "leaf64.cuh"
#include "polymat.cuh"

#include <vector>

namespace pmlg {

namespace {

// H = [A \\ -I]: the bottom block's diagonal constants (the top block is copied in)
__global__ void neg_identity_kernel(uint64_t *H, int64_t n, int64_t hl, uint64_t pm1)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) H[((n + i) * n + i) * hl] = pm1;
}

// flag <- 0 unless the block T[rows n.., cols n..] (T: 2n x 2n, capacity cap) is the identity
__global__ void block_identity_kernel(const uint64_t *__restrict__ T, int64_t n, int64_t cap, int *flag)
{
    const int64_t total = n * n * cap, m = 2 * n;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx / cap, d = idx - e * cap, i = e / n, j = e - i * n;
        const uint64_t want = (i == j && d == 0) ? 1u : 0u;
        if (T[((n + i) * m + (n + j)) * cap + d] != want) atomicExch(flag, 0);
    }
}

// NB[e][d] = (BB[e][d + order] - AS[e][d + order]) mod p, for d < ncap
__global__ void sub_shift_kernel(uint64_t *__restrict__ NB, int64_t ncap, const uint64_t *__restrict__ BB,
                                 int64_t bcap, const uint64_t *__restrict__ AS, int64_t tl, int64_t order,
                                 int64_t ne, uint64_t p)
{
    const int64_t total = ne * ncap;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = idx / ncap, d = idx - e * ncap, k = d + order;
        const uint64_t b = k < bcap ? BB[e * bcap + k] : 0, a = k < tl ? AS[e * tl + k] : 0;
        NB[idx] = b >= a ? b - a : b + p - a;
    }
}

unsigned grid_for(pmlg_ctx *ctx, int64_t work)
{
    const int64_t g = (work + 255) / 256, cap = (int64_t)ctx->sm_count * 8;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

struct DevBuf
{
    cudaStream_t st;
    std::vector<void *> bufs;
    explicit DevBuf(cudaStream_t s) : st(s) {}
    ~DevBuf()
    {
        for (void *b : bufs) cudaFreeAsync(b, st);
    }
    uint64_t *get(int64_t words)
    {
        void *b = nullptr;
        if (cudaMallocAsync(&b, (size_t)(words > 0 ? words : 1) * 8 + 8, st) != cudaSuccess) return nullptr;
        cudaMemsetAsync(b, 0, (size_t)(words > 0 ? words : 1) * 8 + 8, st);
        bufs.push_back(b);
        return (uint64_t *)b;
    }
};

// S (n x n, capacity order + 1) = A^-1 mod x^order; *inv = A(0) invertible
int inv_trunc_device(pmlg_ctx *ctx, uint64_t *S, const uint64_t *A, int64_t n, int64_t alen, int64_t order,
                     uint64_t p, int *inv, cudaStream_t st)
{
    const int64_t m = 2 * n, hl = alen > 0 ? alen : 1, cap = order + 1;
    DevBuf mem(st);
    uint64_t *H = mem.get(m * n * hl), *T = mem.get(m * m * cap);
    int *d_flag = (int *)mem.get(1);
    if (!H || !T || !d_flag) {
        set_error(ctx, "truncated inverse: device allocation failed");
        return PMLG_ENOMEM;
    }
    if (alen > 0) PMLG_CUDA_TRY(cudaMemcpyAsync(H, A, (size_t)(n * n * alen) * 8, cudaMemcpyDeviceToDevice, st));
    neg_identity_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(H, n, hl, p - 1);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    std::vector<int64_t> shift((size_t)m);
    for (int64_t i = 0; i < m; i++) shift[(size_t)i] = i < n ? 0 : order;
    int64_t len = 0;
    PMLG_TRY(pmbasis_device(ctx, T, cap, shift.data(), H, m, n, hl, order, p, &len, st));
    const int one = 1;
    PMLG_CUDA_TRY(cudaMemcpyAsync(d_flag, &one, sizeof(int), cudaMemcpyHostToDevice, st));
    block_identity_kernel<<<grid_for(ctx, n * n * cap), 256, 0, st>>>(T, n, cap, d_flag);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    int h = 0;
    PMLG_CUDA_TRY(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    *inv = h;
    if (h)   // the bottom-left block: row n + i of T begins with its n left entries
        for (int64_t i = 0; i < n; i++)
            PMLG_CUDA_TRY(cudaMemcpyAsync(S + i * n * cap, T + (n + i) * m * cap, (size_t)(n * cap) * 8,
                                          cudaMemcpyDeviceToDevice, st));
    return PMLG_OK;
}

}  // namespace

}  // namespace pmlg

using namespace pmlg;

extern "C" PMLG_API int pmlg_inv_trunc(pmlg_ctx *ctx, uint64_t *S, const uint64_t *A, int64_t n, int64_t alen,
                                       int64_t order, uint64_t p, int *invertible, void *stream)
{
    if (!ctx || n < 0 || alen < 0 || order < 1 || !invertible) return PMLG_EINVAL;
    if (n > 0 && (!S || (alen > 0 && !A))) return PMLG_EINVAL;
    if (2 * n > LEAF64_MAXDIM) {
        set_error(ctx, "truncated inverses support n <= %d (an approximant basis of 2n rows)", LEAF64_MAXDIM / 2);
        return PMLG_EUNSUP;
    }
    if (!h_is_prime(p)) {
        set_error(ctx, "truncated inverses need a prime modulus");
        return PMLG_EBADMOD;
    }
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    *invertible = 0;
    if (n == 0) {
        *invertible = 1;
        return PMLG_OK;
    }
    PMLG_TRY(inv_trunc_device(ctx, S, A, n, alen, order, p, invertible, st));
    PMLG_TRY(device_status(ctx, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    return PMLG_OK;
}

extern "C" PMLG_API int pmlg_dixon(pmlg_ctx *ctx, uint64_t *X, int64_t xcap, const uint64_t *A, const uint64_t *B,
                                   int64_t n, int64_t m, int64_t alen, int64_t blen, int64_t order, int64_t sigma,
                                   uint64_t p, int *ok, void *stream)
{
    if (!ctx || n < 0 || m < 0 || alen < 0 || blen < 0 || order < 1 || sigma < 0 || !ok) return PMLG_EINVAL;
    const int64_t L = (sigma + order - 1) / order;
    if (xcap < L * order || xcap < 1) return PMLG_EINVAL;
    if (n > 0 && m > 0 && (!X || (alen > 0 && !A) || (blen > 0 && !B))) return PMLG_EINVAL;
    if (2 * n > LEAF64_MAXDIM) {
        set_error(ctx, "Dixon lifting supports n <= %d (an approximant basis of 2n rows)", LEAF64_MAXDIM / 2);
        return PMLG_EUNSUP;
    }
    if (!h_is_prime(p)) {
        set_error(ctx, "Dixon lifting needs a prime modulus");
        return PMLG_EBADMOD;
    }
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    *ok = 0;
    if (n == 0) {
        *ok = 1;
        return PMLG_OK;
    }
    const int64_t ne = n * m, ccap = order + 1;
    DevBuf mem(st);
    uint64_t *Cinv = mem.get(n * n * ccap);
    if (!Cinv) return PMLG_ENOMEM;
    int inv = 0;
    PMLG_TRY(inv_trunc_device(ctx, Cinv, A, n, alen, order, p, &inv, st));
    if (!inv) {
        PMLG_CUDA_TRY(cudaStreamSynchronize(st));
        return PMLG_OK;
    }
    if (ne > 0) PMLG_CUDA_TRY(cudaMemsetAsync(X, 0, (size_t)(ne * xcap) * 8, st));
    if (ne > 0) {
        int64_t bcap = blen > 0 ? blen : 1;
        const int64_t tl = (alen > 0 ? alen : 1) + order - 1;
        // the residue never needs more than max(blen, tl) coefficients: two buffers in turn
        const int64_t rcap = bcap > tl ? bcap : tl;
        uint64_t *BB = mem.get(ne * rcap), *NBbuf = mem.get(ne * rcap);
        uint64_t *Sl = mem.get(ne * order);
        uint64_t *AS = mem.get(ne * tl);
        if (!BB || !NBbuf || !Sl || !AS) return PMLG_ENOMEM;
        if (blen > 0) PMLG_CUDA_TRY(cudaMemcpyAsync(BB, B, (size_t)(ne * blen) * 8, cudaMemcpyDeviceToDevice, st));
        // evaluation caches sized for the largest transform and prime count of each product
        // (the middle product needs at most 2 order - 1 points, the product alen + order - 1)
        EvalCache cC, cA;
        {
            CrtPlan pl;
            const int lgC = lg_for(2 * order - 1), lgA = lg_for((alen > 0 ? alen : 1) + order - 1);
            if (lgC <= kMaxLgN && make_plan(ctx, p, lgC, n, order, &pl) == PMLG_OK) {
                cC.words = (size_t)pl.t * ((size_t)1 << lgC) * (size_t)(n * n);
                cC.ea = (uint32_t *)mem.get((int64_t)(cC.words + 1) / 2);
                if (!cC.ea) cC.words = 0;
            }
            if (alen > 0 && lgA <= kMaxLgN &&
                make_plan(ctx, p, lgA, n, alen < order ? alen : order, &pl) == PMLG_OK) {
                cA.words = (size_t)pl.t * ((size_t)1 << lgA) * (size_t)(n * n);
                cA.ea = (uint32_t *)mem.get((int64_t)(cA.words + 1) / 2);
                if (!cA.ea) cA.words = 0;
            }
        }
        for (int64_t l = 0; l * order < sigma; l++) {
            // S = C * BB mod x^order; X += x^(l order) S
            PMLG_TRY(poly_mat_mulmid_device(ctx, Sl, Cinv, BB, n, n, m, ccap, bcap, 0, order, p, st, &cC));
            PMLG_CUDA_TRY(cudaMemcpy2DAsync(X + l * order, (size_t)xcap * 8, Sl, (size_t)order * 8, (size_t)order * 8,
                                            (size_t)ne, cudaMemcpyDeviceToDevice, st));
            // BB = (BB - A S) div x^order
            if (alen > 0) PMLG_TRY(poly_mat_mul_device(ctx, AS, A, Sl, n, n, m, alen, order, p, st, &cA));
            else PMLG_CUDA_TRY(cudaMemsetAsync(AS, 0, (size_t)(ne * tl) * 8, st));
            const int64_t hi = bcap > tl ? bcap : tl;
            const int64_t ncap = hi - order > 0 ? hi - order : 1;
            sub_shift_kernel<<<grid_for(ctx, ne * ncap), 256, 0, st>>>(NBbuf, ncap, BB, bcap, AS, tl, order, ne,
                                                                       p);
            count_launch(ctx);
            PMLG_CUDA_TRY(cudaGetLastError());
            uint64_t *t = BB;
            BB = NBbuf;
            NBbuf = t;
            bcap = ncap;
        }
    }
    *ok = 1;
    PMLG_TRY(device_status(ctx, st));
    PMLG_CUDA_TRY(cudaStreamSynchronize(st));
    return PMLG_OK;
}
