// layout.cu -- the two layouts of a polynomial matrix and the conversions between
// them on the device: entry-major (nmod_poly_mat: entry (i, j) holds its
// coefficients) and coefficient-major (nmod_mat_poly: coefficient k is an r x c
// matrix).  nmod_mat_poly_set_trunc_from_poly_mat
// (flint-extras/src/nmod_mat_poly_extra/nmod_mat_poly_set_from.c:31-52) and
// nmod_poly_mat_set_trunc_from_mat_poly (nmod_poly_mat_extra/nmod_poly_mat_utils.c:185-210).
//
// Both are one tiled transpose of a (entries x coefficients) array: 32 x 32 tiles
// of 64-bit words staged in shared memory (padded rows, no bank conflicts), read
// and written with coalesced accesses, and the padding of the output (the
// coefficients past the truncation) written as zeros in the same pass.  The work
// is pure HBM traffic: 8 bytes read and 8 written per coefficient.
#include "pmlg_internal.cuh"

namespace pmlg {

namespace {

constexpr int TT = 32;          // tile side
constexpr int TROWS = 8;        // thread rows per tile (each thread moves TT / TROWS words)

// out[c * ld_out + r] = (r < rows && c < cols) ? in[r * ld_in + c] : 0, for r < out_cols,
// c < out_rows (the output is out_rows x out_cols, row-major)
__global__ void __launch_bounds__(TT *TROWS)
transpose_pad_kernel(const uint64_t *__restrict__ in, int64_t rows, int64_t cols, int64_t ld_in,
                     uint64_t *__restrict__ out, int64_t out_rows, int64_t out_cols, int64_t ld_out)
{
    __shared__ uint64_t tile[TT][TT + 1];
    const int64_t r0 = (int64_t)blockIdx.x * TT, c0 = (int64_t)blockIdx.y * TT;   // input tile origin
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int k = 0; k < TT; k += TROWS) {
        const int64_t r = r0 + ty + k, c = c0 + tx;
        tile[ty + k][tx] = (r < rows && c < cols) ? in[r * ld_in + c] : 0ull;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TT; k += TROWS) {
        const int64_t c = c0 + ty + k, r = r0 + tx;   // output row c, column r
        if (c < out_rows && r < out_cols) out[c * ld_out + r] = tile[tx][ty + k];
    }
}

int transpose_pad(pmlg_ctx *ctx, const uint64_t *in, int64_t rows, int64_t cols, int64_t ld_in, uint64_t *out,
                  int64_t out_rows, int64_t out_cols, int64_t ld_out, cudaStream_t st)
{
    if (out_rows <= 0 || out_cols <= 0) return PMLG_OK;
    const int64_t gx = (out_cols + TT - 1) / TT, gy = (out_rows + TT - 1) / TT;
    if (gy > 65535) return PMLG_EUNSUP;
    prof_begin(ctx, "layout_transpose", st);
    transpose_pad_kernel<<<dim3((unsigned)gx, (unsigned)gy), dim3(TT, TROWS), 0, st>>>(in, rows, cols, ld_in, out,
                                                                                       out_rows, out_cols, ld_out);
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

}  // namespace

}  // namespace pmlg

using namespace pmlg;

extern "C" PMLG_API int pmlg_poly_mat_to_mat_poly(pmlg_ctx *ctx, uint64_t *out, int64_t out_cap,
                                                  const uint64_t *in, int64_t r, int64_t c, int64_t ld,
                                                  int64_t len, int64_t order, int64_t *out_len, void *stream)
{
    if (!ctx || r < 0 || c < 0 || len < 0 || ld < len || order < 0 || out_cap < 0) return PMLG_EINVAL;
    const int64_t ne = r * c, K = order < len ? order : len;
    if (out_cap < K) return PMLG_EINVAL;
    if ((ne > 0 && K > 0 && !in) || (ne > 0 && out_cap > 0 && !out)) return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    if (ne == 0) {
        if (out_len) *out_len = 0;
        return PMLG_OK;
    }
    // coefficient k of every entry: rows = entries, columns = coefficients [0, K)
    PMLG_TRY(transpose_pad(ctx, in, ne, K, ld, out, out_cap, ne, ne, st));
    if (out_len) {
        // normalised length: the last nonzero coefficient matrix, + 1
        PMLG_TRY(ws_reserve(ctx, &ctx->ws_aux, 256));
        PMLG_TRY(device_max_length(ctx, in, ne, ld, K, (unsigned long long *)ctx->ws_aux.ptr, out_len, st));
    }
    return PMLG_OK;
}

extern "C" PMLG_API int pmlg_mat_poly_to_poly_mat(pmlg_ctx *ctx, uint64_t *out, int64_t out_cap,
                                                  const uint64_t *in, int64_t r, int64_t c, int64_t len,
                                                  int64_t order, void *stream)
{
    if (!ctx || r < 0 || c < 0 || len < 0 || order < 0 || out_cap < 0) return PMLG_EINVAL;
    const int64_t ne = r * c, K = order < len ? order : len;
    if (out_cap < K) return PMLG_EINVAL;
    if ((ne > 0 && K > 0 && !in) || (ne > 0 && out_cap > 0 && !out)) return PMLG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    if (ne == 0) return PMLG_OK;
    // rows = coefficients [0, K), columns = entries; the output entry e gets out_cap coefficients
    return transpose_pad(ctx, in, K, ne, ne, out, ne, out_cap, out_cap, st);
}
