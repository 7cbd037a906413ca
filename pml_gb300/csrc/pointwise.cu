// pointwise.cu -- C_t = A_t * B_t mod q for every evaluation point t.
//
// Two exact forms of the same product (blocks of at most 64 x 64 x 64):
//  * CUDA-core form: 32x32->64-bit multiply-accumulate.  Products are < q^2 <
//    2^60, so eight of them fit in a 64-bit accumulator; after every eight
//    terms the accumulator is folded as hi * (2^32 mod q) + lo (< 2^62 + 2^32),
//    and reduced once at the end.
//  * INT8 tensor-core form: every residue (< 2^30) is split into four 8-bit
//    limbs, a = sum_s a_s 2^(8s).  The 16 limb products A_i * B_j run as
//    mma.sync.m16n8k32 u8 x u8 -> s32 and are summed per weight class
//    s = i + j (at most 4 pairs x 64 terms x 255^2 < 2^24), then recombined
//    as sum_s S_s * (2^(8s) mod q) < 2^57 and reduced mod q on the CUDA cores.
//    (tcgen05 kind::i8 does not exist on sm_103a; mma.sync is the INT8 path.)
#include "pointwise.cuh"

namespace pmlg {

constexpr int PW_PPC = 2;        // evaluation points per CTA
constexpr int PW_THREADS = 256;
constexpr int CC_LD = 68;        // u32 row stride of the CUDA-core smem tiles
constexpr int I8_LD = 80;        // byte row stride of the limb planes (64 + 16 pad)

__device__ __forceinline__ int64_t pw_off(int64_t pt, int64_t e, int lg_tile, int64_t s_tile,
                                          int s_e, int s_p)
{
    const int64_t mask = (1ll << lg_tile) - 1;
    return (pt >> lg_tile) * s_tile + e * s_e + (pt & mask) * s_p;
}

__device__ __forceinline__ int ilog2_small(int x) { return 31 - __clz(x); }

// ---------------------------------------------------------------------------
// CUDA-core form
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(PW_THREADS)
pw_cc_kernel(PwArgs a)
{
    extern __shared__ uint32_t sm[];
    uint32_t *As = sm;                          // [PPC][64][CC_LD]  A[i][l]
    uint32_t *Bs = sm + PW_PPC * 64 * CC_LD;    // [PPC][64][CC_LD]  B[l][j]
    const int tid = threadIdx.x;
    const int lg = ilog2_small(a.pt_tile);
    const int64_t pt0 = (int64_t)blockIdx.x * PW_PPC;

    for (int p = 0; p < PW_PPC; p++) {
        const int64_t pt = pt0 + p;
        const bool valid = pt < a.npts;
        for (int idx = tid; idx < 64 * 64; idx += PW_THREADS) {
            const int i = idx >> 6, l = idx & 63;
            uint32_t va = 0, vb = 0;
            if (valid && i < a.r && l < a.k)
                va = a.A.base[pw_off(pt, (int64_t)i * a.A.ld + l, lg, a.A.s_tile, a.s_e, a.s_p)];
            if (valid && i < a.k && l < a.c)
                vb = a.B.base[pw_off(pt, (int64_t)i * a.B.ld + l, lg, a.B.s_tile, a.s_e, a.s_p)];
            As[(p * 64 + i) * CC_LD + l] = va;
            Bs[(p * 64 + i) * CC_LD + l] = vb;
        }
    }
    __syncthreads();

    const int ti = tid >> 4, tj = tid & 15;
    const int kk = (a.k + 7) & ~7;
    for (int p = 0; p < PW_PPC; p++) {
        const int64_t pt = pt0 + p;
        if (pt >= a.npts) break;
        const uint32_t *Ap = As + p * 64 * CC_LD;
        const uint32_t *Bp = Bs + p * 64 * CC_LD;
        uint64_t acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = 0;
        for (int l0 = 0; l0 < kk; l0 += 8) {
#pragma unroll
            for (int l = l0; l < l0 + 8; l++) {
                uint32_t av[4];
#pragma unroll
                for (int u = 0; u < 4; u++) av[u] = Ap[(4 * ti + u) * CC_LD + l];
                const uint4 bv = *reinterpret_cast<const uint4 *>(&Bp[l * CC_LD + 4 * tj]);
                const uint32_t b4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] += (uint64_t)av[u] * b4[v];
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++)
                    acc[u][v] = (acc[u][v] >> 32) * (uint64_t)a.r32 + (acc[u][v] & 0xffffffffull);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = 4 * ti + u;
            if (i >= a.r) continue;
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const int j = 4 * tj + v;
                if (j >= a.c) continue;
                uint32_t res = mod64_q(acc[u][v], a.q, a.r32, a.r32q, a.oneq);
                const int64_t off = pw_off(pt, (int64_t)i * a.ldc + j, lg, a.s_tile_c, a.s_e, a.s_p);
                if (a.accumulate) {
                    res += a.C[off];
                    res = res >= a.q ? res - a.q : res;
                }
                a.C[off] = res;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// INT8 tensor-core form
// ---------------------------------------------------------------------------

__device__ __forceinline__ void mma_u8(int32_t (&d)[4], const uint32_t (&af)[4], const uint32_t (&bf)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k32.row.col.s32.u8.u8.s32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
        : "r"(af[0]), "r"(af[1]), "r"(af[2]), "r"(af[3]), "r"(bf[0]), "r"(bf[1]));
}

__global__ void __launch_bounds__(PW_THREADS, 1)
pw_i8_kernel(PwArgs a)
{
    extern __shared__ __align__(16) unsigned char sm8[];
    // per point: A limb planes [4][64 rows i][I8_LD] (k contiguous),
    //            B limb planes [4][64 cols j][I8_LD] (B transposed, k contiguous)
    constexpr int PLANE = 64 * I8_LD;
    constexpr int PER_PT = 8 * PLANE;
    const int tid = threadIdx.x;
    const int lg = ilog2_small(a.pt_tile);
    const int64_t pt0 = (int64_t)blockIdx.x * PW_PPC;

    for (int p = 0; p < PW_PPC; p++) {
        const int64_t pt = pt0 + p;
        const bool valid = pt < a.npts;
        unsigned char *Al = sm8 + p * PER_PT;
        unsigned char *Bl = Al + 4 * PLANE;
        for (int idx = tid; idx < 64 * 64; idx += PW_THREADS) {
            const int i = idx >> 6, l = idx & 63;
            uint32_t va = 0, vb = 0;
            if (valid && i < a.r && l < a.k)
                va = a.A.base[pw_off(pt, (int64_t)i * a.A.ld + l, lg, a.A.s_tile, a.s_e, a.s_p)];
            // B element (row i = inner index, col l = output column)
            if (valid && i < a.k && l < a.c)
                vb = a.B.base[pw_off(pt, (int64_t)i * a.B.ld + l, lg, a.B.s_tile, a.s_e, a.s_p)];
#pragma unroll
            for (int s = 0; s < 4; s++) {
                Al[s * PLANE + i * I8_LD + l] = (unsigned char)(va >> (8 * s));
                Bl[s * PLANE + l * I8_LD + i] = (unsigned char)(vb >> (8 * s));
            }
        }
    }
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int kk = (a.k + 31) & ~31;
    // 2 points x 4 m-tiles (16 rows) x 4 n-groups (16 cols) = 32 warp tasks over 8 warps
    for (int task = warp; task < PW_PPC * 16; task += PW_THREADS / 32) {
        const int p = task >> 4, mt = (task >> 2) & 3, ng = task & 3;
        const int64_t pt = pt0 + p;
        if (pt >= a.npts) continue;
        if (mt * 16 >= a.r || ng * 16 >= a.c) continue;
        const unsigned char *Al = sm8 + p * PER_PT;
        const unsigned char *Bl = Al + 4 * PLANE;
        int32_t acc[7][2][4];
#pragma unroll
        for (int s = 0; s < 7; s++)
#pragma unroll
            for (int nt = 0; nt < 2; nt++)
#pragma unroll
                for (int r = 0; r < 4; r++) acc[s][nt][r] = 0;

        for (int ks = 0; ks < kk; ks += 32) {
            uint32_t af[4][4];
#pragma unroll
            for (int s = 0; s < 4; s++) {
                const unsigned char *base = Al + s * PLANE + (mt * 16 + g) * I8_LD + ks + tig * 4;
                af[s][0] = *reinterpret_cast<const uint32_t *>(base);
                af[s][1] = *reinterpret_cast<const uint32_t *>(base + 8 * I8_LD);
                af[s][2] = *reinterpret_cast<const uint32_t *>(base + 16);
                af[s][3] = *reinterpret_cast<const uint32_t *>(base + 8 * I8_LD + 16);
            }
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                uint32_t bf[4][2];
#pragma unroll
                for (int s = 0; s < 4; s++) {
                    const unsigned char *base = Bl + s * PLANE + (ng * 16 + nt * 8 + g) * I8_LD + ks + tig * 4;
                    bf[s][0] = *reinterpret_cast<const uint32_t *>(base);
                    bf[s][1] = *reinterpret_cast<const uint32_t *>(base + 16);
                }
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) mma_u8(acc[i + j][nt], af[i], bf[j]);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 2; nt++)
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int i = mt * 16 + g + ((r >> 1) << 3);
                const int j = ng * 16 + nt * 8 + tig * 2 + (r & 1);
                if (i >= a.r || j >= a.c) continue;
                uint64_t v = 0;
#pragma unroll
                for (int s = 0; s < 7; s++) v += (uint64_t)(uint32_t)acc[s][nt][r] * a.w8[s];
                uint32_t res = mod64_q(v, a.q, a.r32, a.r32q, a.oneq);
                const int64_t off = pw_off(pt, (int64_t)i * a.ldc + j, lg, a.s_tile_c, a.s_e, a.s_p);
                if (a.accumulate) {
                    res += a.C[off];
                    res = res >= a.q ? res - a.q : res;
                }
                a.C[off] = res;
            }
    }
}

// ---------------------------------------------------------------------------
// CUDA-core form, pipelined: a persistent CTA of 512 threads walks over pairs
// of points; 256 threads compute each point (4 x 4 outputs per thread) while
// cp.async brings the next pair into the other half of a two-stage shared
// memory ring, so global loads overlap the multiply-accumulate.
// ---------------------------------------------------------------------------

constexpr int CC2_THREADS = 512;
constexpr int CC2_PLANE = 64 * CC_LD;                 // one 64 x 64 matrix, padded rows
constexpr int CC2_STAGE = 2 * 2 * CC2_PLANE;          // 2 points x (A, B)

__device__ __forceinline__ void cp_async4(uint32_t *smem_dst, const uint32_t *gsrc)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

__global__ void __launch_bounds__(CC2_THREADS, 1)
pw_cc2_kernel(PwArgs a)
{
    extern __shared__ uint32_t sm[];
    const int tid = threadIdx.x;
    const int lg = ilog2_small(a.pt_tile);
    const int64_t items = (a.npts + 1) >> 1;

    // zero both stages once: the padding outside r x k / k x c stays zero
    for (int idx = tid; idx < 2 * CC2_STAGE; idx += CC2_THREADS) sm[idx] = 0;
    __syncthreads();

    auto issue = [&](int64_t item, int stage) {
        uint32_t *base = sm + stage * CC2_STAGE;
        const int64_t pt0 = item * 2;
        for (int idx = tid; idx < 2 * 4096; idx += CC2_THREADS) {
            const int p = idx >> 12, e = idx & 4095, i = e >> 6, l = e & 63;
            const int64_t pt = pt0 + p;
            if (pt >= a.npts) continue;
            uint32_t *As = base + p * 2 * CC2_PLANE;
            uint32_t *Bs = As + CC2_PLANE;
            if (i < a.r && l < a.k)
                cp_async4(&As[i * CC_LD + l], &a.A.base[pw_off(pt, (int64_t)i * a.A.ld + l, lg, a.A.s_tile, a.s_e, a.s_p)]);
            if (i < a.k && l < a.c)
                cp_async4(&Bs[i * CC_LD + l], &a.B.base[pw_off(pt, (int64_t)i * a.B.ld + l, lg, a.B.s_tile, a.s_e, a.s_p)]);
        }
    };

    const int pl = tid >> 8, ltid = tid & 255, ti = ltid >> 4, tj = ltid & 15;
    const int kk = (a.k + 7) & ~7;
    int64_t item = blockIdx.x;
    if (item < items) issue(item, 0);
    cp_async_commit();
    int stage = 0;
    for (; item < items; item += gridDim.x, stage ^= 1) {
        const int64_t next = item + gridDim.x;
        if (next < items) issue(next, stage ^ 1);
        cp_async_commit();
        cp_async_wait1();
        __syncthreads();

        const int64_t pt = item * 2 + pl;
        if (pt < a.npts) {
            const uint32_t *Ap = sm + stage * CC2_STAGE + pl * 2 * CC2_PLANE;
            const uint32_t *Bp = Ap + CC2_PLANE;
            uint64_t acc[4][4];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] = 0;
            for (int l0 = 0; l0 < kk; l0 += 8) {
#pragma unroll
                for (int l = l0; l < l0 + 8; l++) {
                    uint32_t av[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) av[u] = Ap[(4 * ti + u) * CC_LD + l];
                    const uint4 bv = *reinterpret_cast<const uint4 *>(&Bp[l * CC_LD + 4 * tj]);
                    const uint32_t b4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int v = 0; v < 4; v++) acc[u][v] += (uint64_t)av[u] * b4[v];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int v = 0; v < 4; v++)
                        acc[u][v] = (acc[u][v] >> 32) * (uint64_t)a.r32 + (acc[u][v] & 0xffffffffull);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int i = 4 * ti + u;
                if (i >= a.r) continue;
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const int j = 4 * tj + v;
                    if (j >= a.c) continue;
                    uint32_t res = mod64_q(acc[u][v], a.q, a.r32, a.r32q, a.oneq);
                    const int64_t off = pw_off(pt, (int64_t)i * a.ldc + j, lg, a.s_tile_c, a.s_e, a.s_p);
                    if (a.accumulate) {
                        res += a.C[off];
                        res = res >= a.q ? res - a.q : res;
                    }
                    a.C[off] = res;
                }
            }
        }
        __syncthreads();   // this stage is refilled two items later
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

void pointwise_set_modulus(PwArgs &a, uint32_t q)
{
    a.q = q;
    a.r32 = (uint32_t)((1ull << 32) % q);
    a.r32q = h_shoup_q(a.r32, q);
    a.oneq = (uint32_t)((1ull << 32) / q);
    uint64_t w = 1;
    for (int s = 0; s < 7; s++) {
        a.w8[s] = (uint32_t)(w % q);
        w = (w << 8) % q;
    }
}

static int form_resolve(int form)
{
    return form == PMLG_FORM_AUTO ? PMLG_FORM_CUDA_CORE : form;
}

int pointwise_launch(pmlg_ctx *ctx, const PwArgs &a, int form, cudaStream_t st)
{
    static bool attr_done = false;
    const size_t smem_i8 = (size_t)PW_PPC * 8 * 64 * I8_LD;
    const size_t smem_cc2 = 2ull * CC2_STAGE * sizeof(uint32_t);
    if (!attr_done) {
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_i8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_i8));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_cc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cc2));
        attr_done = true;
    }
    if (a.npts <= 0) return PMLG_OK;
    const int64_t grid = (a.npts + PW_PPC - 1) / PW_PPC;
    if (grid > 0x7fffffffll) return PMLG_EUNSUP;
    if (form_resolve(form) == PMLG_FORM_INT8_TC) {
        prof_begin(ctx, "pointwise_int8_tc", st);
        pw_i8_kernel<<<(unsigned)grid, PW_THREADS, smem_i8, st>>>(a);
    } else {
        const int64_t items = (a.npts + 1) / 2;
        const int64_t g2 = items < ctx->sm_count ? items : ctx->sm_count;
        prof_begin(ctx, "pointwise_cuda_core", st);
        pw_cc2_kernel<<<(unsigned)g2, CC2_THREADS, smem_cc2, st>>>(a);
    }
    prof_end(ctx, st);
    count_launch(ctx);
    PMLG_CUDA_TRY(cudaGetLastError());
    return PMLG_OK;
}

int pointwise_blocked(pmlg_ctx *ctx, PwArgs a, int64_t r, int64_t k, int64_t c, int form,
                      cudaStream_t st)
{
    const PwArgs base = a;
    for (int64_t ib = 0; ib < r; ib += 64)
        for (int64_t jb = 0; jb < c; jb += 64)
            for (int64_t kb = 0; kb < k; kb += 64) {
                PwArgs b = base;
                b.r = (int)((r - ib) < 64 ? (r - ib) : 64);
                b.c = (int)((c - jb) < 64 ? (c - jb) : 64);
                b.k = (int)((k - kb) < 64 ? (k - kb) : 64);
                b.A.base = base.A.base + (ib * base.A.ld + kb) * base.s_e;
                b.B.base = base.B.base + (kb * base.B.ld + jb) * base.s_e;
                b.C = base.C + (ib * base.ldc + jb) * base.s_e;
                b.accumulate = base.accumulate || kb > 0;
                PMLG_TRY(pointwise_launch(ctx, b, form, st));
            }
    return PMLG_OK;
}

}  // namespace pmlg

using namespace pmlg;

extern "C" PMLG_API int pmlg_nmod_mat_mul_batch_u32(pmlg_ctx *ctx, uint32_t *C, const uint32_t *A,
                                                    const uint32_t *B, int64_t nbatch, int64_t r,
                                                    int64_t k, int64_t c, uint64_t p, void *stream)
{
    if (!ctx || nbatch < 0 || r < 0 || k < 0 || c < 0) return PMLG_EINVAL;
    if (nbatch == 0 || r == 0 || c == 0) return PMLG_OK;
    if (!A || !B || !C) return PMLG_EINVAL;
    if (p < 2 || p >= (1ull << 30)) {
        set_error(ctx, "batched matrix product needs 2 <= p < 2^30");
        return PMLG_EBADMOD;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (k == 0)
        return cudaMemsetAsync(C, 0, (size_t)(nbatch * r * c) * sizeof(uint32_t), st) == cudaSuccess
                   ? PMLG_OK : PMLG_ECUDA;
    PMLG_CUDA_TRY(cudaSetDevice(ctx->device));
    PwArgs a{};
    a.A = {A, r * k, k};
    a.B = {B, k * c, c};
    a.C = C;
    a.s_tile_c = r * c;
    a.ldc = c;
    a.pt_tile = 1;
    a.s_e = 1;
    a.s_p = 0;
    a.npts = nbatch;
    a.accumulate = 0;
    pointwise_set_modulus(a, (uint32_t)p);
    return pointwise_blocked(ctx, a, r, k, c, ctx->form, st);
}
