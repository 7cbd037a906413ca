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
#include "ntt.cuh"

#include <cuda_fp16.h>

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
                uint32_t res = mod64_q(v, a.q, a.r32, a.r32q, a.oneq);   // w8 carries the output scale
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
                    res = reduce_once(shoup_mul(res, a.scale, a.scaleq, a.q), a.q);
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
// FP16-digit tensor-core form (tcgen05.mma kind::f16, FP32 accumulators in TMEM)
// ---------------------------------------------------------------------------
//
// Residues are written in balanced digits (B entries centred first, |x| < q/2 < 2^29):
//   A entries: 4 digits base 2^8,  |d_i| <= 128 ;  B entries: 3 digits base 2^10, |e_j| <= 512.
// All digits are exact in FP16, every product d_i e_j is at most 2^16 in size,
// and a sum over the 64 inner indices at most 2^22, so the FP32 accumulation
// of the tensor cores is exact at every step (integers of at most 2^22).
//
// Per point the MMAs compute all 12 digit products S_ij = A_i B_j; the
// epilogue recombines C = sum_ij S_ij 2^(8i + 10j) mod q on the CUDA cores.
// The A operand is stacked two digits high (M = 128: rows 0..63 digit 2s,
// rows 64..127 digit 2s+1, stack s = 0, 1), the B operand holds the three
// digits side by side.  The output columns are split into two regions
// (columns 0..31 and 32..63), each with its own TMEM range and mbarriers, so
// the MMAs of the next point fill one region while the epilogue still reads
// the other:  region h = 2 stacks x (N = 96 = 3 digits x 32 columns).
//
// The CTA is warp-specialised (one CTA per SM, points taken in pairs):
//   warps 0..7   epilogue: tcgen05.ld, integer recombination, reduction mod q,
//                staging in shared memory, coalesced write of the pair;
//   warps 8..15  loads of a point pair (the two points share 8 bytes in the
//                point-tiled layout) and the digit split into two stages;
//   warp 16      one thread issues the MMAs of a point into each region as
//                soon as it is drained, and commits to the mbarriers.
// Digits reach FP16 without conversion instructions: 0x6400 + u is the FP16
// encoding of 1024 + u for 0 <= u <= 1024, and one packed subtraction removes
// the bias.  The FP32 sums come back as integers the same way: a first MMA
// with constant operands puts 1.5 * 2^23 into every accumulator, and for
// |S| <= 2^22 the encoding of 1.5 * 2^23 + S is 0x4B400000 + S (every partial
// sum stays an integer in [2^23, 2^24], exact in FP32).
// Every mbarrier wait is bounded; a wait that gives up raises a shared abort
// flag that turns every later wait into a no-op, so all warps leave their
// loops, the MMAs in flight are drained and the kernel records the error.

constexpr int F16_EPI_WARPS = 8;
constexpr int F16_SPLIT_WARPS = 8;
constexpr int F16_MMA_WARP = F16_EPI_WARPS + F16_SPLIT_WARPS;
constexpr int F16_THREADS = (F16_MMA_WARP + 1) * 32;
constexpr int F16_A_BYTES = 128 * 64 * 2;            // one stack: M = 128 x K = 64, FP16
constexpr int F16_B_BYTES = 192 * 64 * 2;            // N = 2 regions x 96, K = 64
constexpr int F16_STAGE = 2 * F16_A_BYTES + F16_B_BYTES;
constexpr int F16_CST_LD = 68;                       // padded staging row (words): conflict-free v4 stores
constexpr int F16_CST_WORDS = 64 * F16_CST_LD;       // one (point, digit parity) plane
constexpr int F16_BIAS_A = 128 * 16 * 2, F16_BIAS_B = 96 * 16 * 2;   // constant bias operands (K = 16)
constexpr int F16_SMEM = 2 * F16_STAGE + 4 * F16_CST_WORDS * 4 + F16_BIAS_A + F16_BIAS_B + 1024;   // + alignment slack
constexpr uint32_t F16_TMEM_COLS = 512;
#ifndef PMLG_F16_SUSPEND_NS
#define PMLG_F16_SUSPEND_NS 0
#endif
constexpr uint32_t F16_SUSPEND_NS = PMLG_F16_SUSPEND_NS;   // suspend-time hint per poll (0: none)
constexpr uint64_t F16_WAIT_NS = 500000000ull;       // give up after 0.5 s; a legitimate wait lasts microseconds

__device__ __forceinline__ uint32_t canon_off(int row, int k)
{
    // byte offset of (row, k) in a K-major no-swizzle tile with K = 64 (2-byte elements)
    return (uint32_t)((row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t sbo = 1024)
{
    // start address, LBO = 128 B (next core matrix along K), SBO (next 8 rows; 1024 B for
    // K = 64 tiles), descriptor version 1, no swizzle
    return (uint64_t)((saddr >> 4) & 0x3fff) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(b)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t *b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"((uint32_t)__cvta_generic_to_shared(b)) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase of the given parity; false when it gave up (or
// another warp already did), in which case the abort flag is set.  With a
// suspend-time hint the thread sleeps inside try_wait until the phase
// completes or the hint expires.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile int *abort)
{
    const uint32_t addr = (uint32_t)__cvta_generic_to_shared(b);
    uint64_t t0 = 0;
    for (int it = 0; it < (1 << 30); it++) {
        uint32_t done;
        if (F16_SUSPEND_NS)
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.u32 %0, 1, 0, p;\n}"
                         : "=r"(done) : "r"(addr), "r"(parity), "r"(F16_SUSPEND_NS) : "memory");
        else
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                         : "=r"(done) : "r"(addr), "r"(parity) : "memory");
        if (done) return true;
        if ((it & 63) == 0) {
            if (abort && *abort) return false;
            const uint64_t now = globaltimer_ns();
            if (it == 0)
                t0 = now;
            else if (now - t0 > F16_WAIT_NS)
                break;
        }
    }
    if (abort) *abort = 1;
    return false;
}

__device__ __forceinline__ void tc_commit(uint64_t *b)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"((uint32_t)__cvta_generic_to_shared(b)) : "memory");
}

// Digit planes of two A entries (same row, adjacent K) as half2 words, digit
// i in word i.  With y = x + 0x80808080 (x < 2^30) the bytes b_i of y give
// x = sum (b_i - 128) 256^i, |b_i - 128| <= 128; 0x6400 + b is the FP16
// encoding of 1024 + b, and one packed subtraction of 1152 leaves b - 128.
__device__ __forceinline__ void a_digit_pairs(uint32_t x0, uint32_t x1, uint32_t (&w)[4])
{
    const uint32_t y0 = x0 + 0x80808080u, y1 = x1 + 0x80808080u;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t sel = (uint32_t)(i | (i << 4) | ((4 + i) << 8) | ((4 + i) << 12));
        const uint32_t b = (__byte_perm(y0, y1, sel) & 0x00ff00ffu) | 0x64006400u;
        asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(w[i]) : "r"(b), "r"(0x64806480u));
    }
}

// Balanced base-2^10 digit planes of two B entries as half2 words.  The
// centred residue t lies in (-2^29, 2^29), so y = t + 512 (1 + 2^10 + 2^20) has
// two 10-bit fields f_0, f_1 and an 11-bit top field f_2 <= 1024 with
// t = sum (f_j - 512) 2^(10 j); the encodings 0x6400 + f_j reach 0x6800 at
// most (an addition, not an or, for the top field), minus 1536 gives f_j - 512.
__device__ __forceinline__ void b_digit_pairs(uint32_t x0, uint32_t x1, uint32_t q, uint32_t (&w)[3])
{
    const uint32_t h = q >> 1;
    const uint32_t y0 = x0 + 0x20080200u - (x0 > h ? q : 0u);
    const uint32_t y1 = x1 + 0x20080200u - (x1 > h ? q : 0u);
    uint32_t b[3];
    b[0] = (__byte_perm(y0, y1, 0x5410) & 0x03ff03ffu) | 0x64006400u;
    b[1] = ((__byte_perm(y0, y1, 0x6521) >> 2) & 0x03ff03ffu) | 0x64006400u;
    b[2] = ((__byte_perm(y0, y1, 0x7632) >> 4) & 0x07ff07ffu) + 0x64006400u;
#pragma unroll
    for (int j = 0; j < 3; j++) asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(w[j]) : "r"(b[j]), "r"(0x66006600u));
}

// x mod q up to one multiple of q: x < 2^64, result in [0, 2q)
__device__ __forceinline__ uint32_t mod64_q_2(uint64_t x, uint32_t q, uint32_t r32, uint32_t r32q, uint32_t oneq)
{
    const uint32_t t = shoup_mul((uint32_t)(x >> 32), r32, r32q, q);   // [0, 2q)
    const uint32_t l = shoup_mul((uint32_t)x, 1u, oneq, q);             // [0, 2q)
    const uint32_t s = t + l;                                           // < 4q < 2^32
    return min(s, s - 2 * q);
}

#define TC_LD16(taddr, v)                                                                                       \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),     \
                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]) \
                 : "r"(taddr))

// values of entry e at points pt0 and pt0 + 1
template <bool TILE>
__device__ __forceinline__ uint2 f16_load_pair(const PwOperand &op, int64_t e, int64_t pt0, bool has1, int lg,
                                               const PwArgs &a)
{
    if (TILE)   // point-tiled layout, pt0 even: the two values are adjacent
        return __ldg(reinterpret_cast<const uint2 *>(op.base + ((pt0 / kPtTile) * op.s_tile + e * kPtTile +
                                                                (pt0 % kPtTile))));
    uint2 v;
    v.x = op.base[pw_off(pt0, e, lg, op.s_tile, a.s_e, a.s_p)];
    v.y = has1 ? op.base[pw_off(pt0 + 1, e, lg, op.s_tile, a.s_e, a.s_p)] : 0u;
    return v;
}

template <bool TILE, bool PACK, bool SKIP>
__global__ void __launch_bounds__(F16_THREADS, 1)
pw_f16_kernel(PwArgs a)
{
    extern __shared__ __align__(16) unsigned char f16_raw[];
    // 1024-byte aligned start, by pointer arithmetic on the shared array (the
    // accesses stay shared-memory instructions)
    unsigned char *sm = f16_raw + ((1024u - ((uint32_t)__cvta_generic_to_shared(f16_raw) & 1023u)) & 1023u);
    uint32_t *Cst = (uint32_t *)(sm + 2 * F16_STAGE);
    __shared__ __align__(8) uint64_t full[2], empty[2], tfull[2], tempty[2], drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lg = ilog2_small(a.pt_tile);
    const uint32_t q = a.q;
    // Small blocks are packed: 64 >> lmt points share one MMA problem as the
    // diagonal blocks of block-diagonal 64 x 64 operands (the other blocks are
    // zero), so a unit of 2 * (64 >> lmt) consecutive points fills both stages.
    const int lmt = PACK ? a.lmt : 6, mt = 1 << lmt, G = 64 >> lmt;
    const int64_t nunits = (a.npts + 2 * G - 1) / (2 * G);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"((uint32_t)__cvta_generic_to_shared(&tmem_slot)), "r"(F16_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // Bias operands: every entry of A is 256 and of B 3072 (both exact in FP16), so one
    // K = 16 MMA puts 16 x 256 x 3072 = 1.5 x 2^23 into every accumulator before the digit
    // products; the sums then come back as integers straight from their FP32 bits
    // (0x4B400000 + S for |S| <= 2^22).
    {
        uint32_t *bias = reinterpret_cast<uint32_t *>(sm + 2 * F16_STAGE + 4 * F16_CST_WORDS * 4);
        for (int i = tid; i < (F16_BIAS_A + F16_BIAS_B) / 4; i += blockDim.x)
            bias[i] = i < F16_BIAS_A / 4 ? 0x5C005C00u : 0x6A006A00u;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(&full[s], F16_SPLIT_WARPS);
            mbar_init(&empty[s], 1);
            mbar_init(&tfull[s], 1);
            mbar_init(&tempty[s], F16_EPI_WARPS);
        }
        mbar_init(&drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_abort = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    volatile int *abort = &s_abort;

    if (warp >= F16_EPI_WARPS && warp < F16_MMA_WARP) {
        // ---- loads and digit split: one warp writes one 8 x 8 core matrix per item
        const int sw = warp - F16_EPI_WARPS;
        const int row_in = lane >> 2, kp = lane & 3;
        int lc = 0;
        for (int64_t gc = blockIdx.x; gc < nunits; gc += gridDim.x, lc++) {
            const int64_t pt0 = 2 * G * gc;
            uint2 va[8][2], vb[8][2];
#pragma unroll
            for (int itn = 0; itn < 8; itn++) {
                const int cmi = sw + 8 * itn;
                const int i = (cmi >> 3) * 8 + row_in, l = (cmi & 7) * 8 + 2 * kp;
                const uint2 z = make_uint2(0u, 0u);
                if constexpr (!PACK) {
                    const bool has1 = pt0 + 1 < a.npts;
                    va[itn][0] = (i < a.r && l < a.k) ? f16_load_pair<TILE>(a.A, (int64_t)i * a.A.ld + l, pt0, has1, lg, a) : z;
                    va[itn][1] = (i < a.r && l + 1 < a.k) ? f16_load_pair<TILE>(a.A, (int64_t)i * a.A.ld + l + 1, pt0, has1, lg, a) : z;
                    vb[itn][0] = (i < a.c && l < a.k) ? f16_load_pair<TILE>(a.B, (int64_t)l * a.B.ld + i, pt0, has1, lg, a) : z;
                    vb[itn][1] = (i < a.c && l + 1 < a.k) ? f16_load_pair<TILE>(a.B, (int64_t)(l + 1) * a.B.ld + i, pt0, has1, lg, a) : z;
                } else {
                    // block (g, gl) of A holds point pair g when g == gl; B likewise with (gn, gl)
                    const int g = i >> lmt, gl = l >> lmt, ii = i & (mt - 1), ll = l & (mt - 1);
                    const int64_t pA = pt0 + 2 * g;
                    const bool okA = g == gl && ii < a.r && pA < a.npts, okB = g == gl && ii < a.c && pA < a.npts;
                    const bool h1 = pA + 1 < a.npts;
                    va[itn][0] = (okA && ll < a.k) ? f16_load_pair<TILE>(a.A, (int64_t)ii * a.A.ld + ll, pA, h1, lg, a) : z;
                    va[itn][1] = (okA && ll + 1 < a.k) ? f16_load_pair<TILE>(a.A, (int64_t)ii * a.A.ld + ll + 1, pA, h1, lg, a) : z;
                    vb[itn][0] = (okB && ll < a.k) ? f16_load_pair<TILE>(a.B, (int64_t)ll * a.B.ld + ii, pA, h1, lg, a) : z;
                    vb[itn][1] = (okB && ll + 1 < a.k) ? f16_load_pair<TILE>(a.B, (int64_t)(ll + 1) * a.B.ld + ii, pA, h1, lg, a) : z;
                }
            }
#pragma unroll
            for (int pp = 0; pp < 2; pp++) {
                if (mbar_wait(&empty[pp], (uint32_t)((lc & 1) ^ 1), abort)) {
                    unsigned char *A01 = sm + pp * F16_STAGE;
                    unsigned char *Bc = A01 + 2 * F16_A_BYTES;
#pragma unroll
                    for (int itn = 0; itn < 8; itn++) {
                        const int cmi = sw + 8 * itn;
                        const int i = (cmi >> 3) * 8 + row_in, l = (cmi & 7) * 8 + 2 * kp;
                        uint32_t wa[4], wb[3];
                        a_digit_pairs(pp ? va[itn][0].y : va[itn][0].x, pp ? va[itn][1].y : va[itn][1].x, wa);
#pragma unroll
                        for (int d = 0; d < 4; d++)
                            *reinterpret_cast<uint32_t *>(A01 + (d >> 1) * F16_A_BYTES + canon_off((d & 1) * 64 + i, l)) = wa[d];
                        b_digit_pairs(pp ? vb[itn][0].y : vb[itn][0].x, pp ? vb[itn][1].y : vb[itn][1].x, q, wb);
                        const int rb = 96 * (i >> 5) + (i & 31);    // B row of output column i, digit 0
#pragma unroll
                        for (int j = 0; j < 3; j++)
                            *reinterpret_cast<uint32_t *>(Bc + canon_off(rb + 32 * j, l)) = wb[j];
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[pp]);
            }
        }
    } else if (warp == F16_MMA_WARP) {
        // ---- MMA issue (one thread)
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | ((uint32_t)(96 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
            const uint32_t bias_a = (uint32_t)__cvta_generic_to_shared(sm + 2 * F16_STAGE + 4 * F16_CST_WORDS * 4);
            const uint64_t dba = umma_desc(bias_a, 256), dbb = umma_desc(bias_a + F16_BIAS_A, 256);
            uint32_t p = 0;
            int lc = 0;
            for (int64_t gc = blockIdx.x; gc < nunits; gc += gridDim.x, lc++) {
                for (int pp = 0; pp < 2; pp++, p++) {
                    bool ok = mbar_wait(&full[pp], (uint32_t)(lc & 1), abort);
                    const uint32_t base = (uint32_t)__cvta_generic_to_shared(sm + pp * F16_STAGE);
                    for (int h = 0; h < 2; h++) {
                        ok = ok && mbar_wait(&tempty[h], (p & 1) ^ 1, abort);   // region h of point p - 1 drained
                        if (!ok) break;
                        asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            // the bias first (overwriting the accumulators), then the digit products
                            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                                         ::"r"(tmem + (uint32_t)(256 * h + 96 * s)), "l"(dba), "l"(dbb), "r"(idesc),
                                           "r"(0u));
#pragma unroll
                            for (int ks = 0; ks < 4; ks++) {
                                const uint64_t da = umma_desc(base + s * F16_A_BYTES + ks * 256);
                                const uint64_t db = umma_desc(base + 2 * F16_A_BYTES + h * 12 * 1024 + ks * 256);
                                asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                                             ::"r"(tmem + (uint32_t)(256 * h + 96 * s)), "l"(da), "l"(db), "r"(idesc),
                                               "r"(1u));
                            }
                        }
                        tc_commit(&tfull[h]);
                    }
                    if (ok) tc_commit(&empty[pp]);
                }
            }
            // every MMA issued has completed before TMEM is released
            tc_commit(&drain);
            if (!mbar_wait(&drain, 0, nullptr)) *abort = 1;
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w reads TMEM lanes 32 (w & 3) + lane, columns half (w >> 2) of each region
        const int sp = warp & 3, ch = warp >> 2, hi = sp >> 1;
        const int i = (32 * sp + lane) & 63;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * sp) << 16);
        uint32_t w[2][3];
        uint64_t koff = a.negoff;
#pragma unroll
        for (int s = 0; s < 2; s++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                w[s][j] = a.wd[2 * s + hi][j];
                koff -= 0x4B400000ull * w[s][j];
            }
        // This warp's outputs in region h are rows 32 (sp & 1) + [0, 32) and columns
        // 32h + 16ch + [0, 16).  Packed blocks (2^lmt <= 32) have their diagonal outputs
        // of region h in rows 32h..32h+31, so only warps with (sp & 1) == h hold any;
        // unpacked, the warp holds some only when its rows and columns meet the r x c
        // result.  With SKIP (every shape below 64 x 64) a warp without any skips the
        // region but still waits for it and reports it drained, so every mbarrier phase
        // keeps its arrival count; the write-out reads only outputs that are in the result.
        // Unpacked with SKIP, the two warps of a lane quarter swap their 16-column halves
        // from one point to the next: with 3 of the 4 column granules in the result (33 to
        // 48 columns) each then computes 3 granules per two points instead of 4 and 2.
        const bool packed = lmt < 6;
        const bool alt = SKIP && !packed;
        uint32_t p = 0;
        for (int64_t gc = blockIdx.x; gc < nunits; gc += gridDim.x) {
            for (int pp = 0; pp < 2; pp++, p++) {
                uint32_t *row = Cst + (pp * 2 + hi) * F16_CST_WORDS + i * F16_CST_LD;
                const int chp = alt ? ch ^ (int)(p & 1u) : ch;
                const bool use0 = !SKIP || (packed ? (sp & 1) == 0 : 32 * (sp & 1) < a.r && 16 * chp < a.c);
                const bool use1 = !SKIP || (packed ? (sp & 1) == 1 : 32 * (sp & 1) < a.r && 32 + 16 * chp < a.c);
                for (int h = 0; h < 2; h++) {
                    const bool useful = h ? use1 : use0;
                    uint64_t acc[16];
#pragma unroll
                    for (int u = 0; u < 16; u++) acc[u] = 0;
                    if (mbar_wait(&tfull[h], p & 1, abort) && useful) {
                        asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            uint32_t v[3][16];
#pragma unroll
                            for (int j = 0; j < 3; j++)
                                TC_LD16(lane_base + (uint32_t)(256 * h + 96 * s + 32 * j + 16 * chp), v[j]);
                            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                            for (int j = 0; j < 3; j++)
#pragma unroll
                                for (int u = 0; u < 16; u++)
                                    acc[u] += (uint64_t)v[j][u] * w[s][j];   // bits = 0x4B400000 + S
                        }
                        asm volatile("tcgen05.fence::before_thread_sync;");
                    }
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[h]);
                    if (useful) {
                        uint32_t r[16];
#pragma unroll
                        for (int u = 0; u < 16; u++) r[u] = mod64_q_2(acc[u] + koff, q, a.r32, a.r32q, a.oneq);
#pragma unroll
                        for (int m = 0; m < 4; m++)
                            *reinterpret_cast<uint4 *>(row + 32 * h + 16 * chp + 4 * m) =
                                make_uint4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
                    }
                }
            }
            asm volatile("bar.sync 1, %0;" ::"n"(F16_EPI_WARPS * 32) : "memory");
            // write the unit: lanes along the entries of a row; output (i, n) of the
            // diagonal block g is entry (i, n) mod mt of points pt0 + 2g (+1)
            const int64_t pt0base = 2 * G * gc;
            const bool has1base = pt0base + 1 < a.npts;
#pragma unroll 4
            for (int m = 0; m < 16; m++) {
                const int e = tid + F16_EPI_WARPS * 32 * m;
                const int i2 = e >> 6, n2 = e & 63;
                int ii = i2, n = n2;
                int64_t pt0 = pt0base;
                bool has1 = has1base;
                if constexpr (PACK) {
                    const int g = i2 >> lmt;
                    ii = i2 & (mt - 1);
                    n = n2 & (mt - 1);
                    pt0 = pt0base + 2 * g;
                    if ((n2 >> lmt) != g || pt0 >= a.npts) continue;
                    has1 = pt0 + 1 < a.npts;
                }
                if (ii >= a.r || n >= a.c) continue;
                const int o = i2 * F16_CST_LD + n2;
                // the two digit-parity halves, each in [0, 2q)
                uint32_t v0 = Cst[o] + Cst[F16_CST_WORDS + o];
                uint32_t v1 = Cst[2 * F16_CST_WORDS + o] + Cst[3 * F16_CST_WORDS + o];
                v0 = min(v0, v0 - 2 * q);
                v1 = min(v1, v1 - 2 * q);
                v0 = v0 >= q ? v0 - q : v0;
                v1 = v1 >= q ? v1 - q : v1;
                const int64_t ce = (int64_t)ii * a.ldc + n;
                if (TILE) {
                    uint2 *dst = reinterpret_cast<uint2 *>(a.C + ((pt0 / kPtTile) * a.s_tile_c + ce * kPtTile +
                                                                  (pt0 % kPtTile)));
                    if (a.accumulate) {
                        const uint2 old = *dst;
                        v0 += old.x;
                        v1 += old.y;
                        v0 = v0 >= q ? v0 - q : v0;
                        v1 = v1 >= q ? v1 - q : v1;
                    }
                    *dst = make_uint2(v0, v1);
                } else {
                    uint32_t *d0 = a.C + pw_off(pt0, ce, lg, a.s_tile_c, a.s_e, a.s_p);
                    if (a.accumulate) {
                        v0 += *d0;
                        v0 = v0 >= q ? v0 - q : v0;
                    }
                    *d0 = v0;
                    if (has1) {
                        uint32_t *d1 = a.C + pw_off(pt0 + 1, ce, lg, a.s_tile_c, a.s_e, a.s_p);
                        if (a.accumulate) {
                            v1 += *d1;
                            v1 = v1 >= q ? v1 - q : v1;
                        }
                        *d1 = v1;
                    }
                }
            }
            asm volatile("bar.sync 2, %0;" ::"n"(F16_EPI_WARPS * 32) : "memory");
        }
    }

    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && s_abort && a.err) atomicExch(a.err, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(F16_TMEM_COLS));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

void pointwise_set_modulus(PwArgs &a, uint32_t q, uint32_t scale)
{
    a.q = q;
    a.r32 = (uint32_t)((1ull << 32) % q);
    a.r32q = h_shoup_q(a.r32, q);
    a.oneq = (uint32_t)((1ull << 32) / q);
    a.scale = scale % q;
    a.scaleq = h_shoup_q(a.scale, q);
    // the recombination weights of the tensor-core forms carry the scale for free
    uint64_t w = a.scale;
    for (int s = 0; s < 7; s++) {
        a.w8[s] = (uint32_t)w;
        w = (w << 8) % q;
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 3; j++)
            a.wd[i][j] = (uint32_t)((unsigned __int128)h_powmod(2, (uint64_t)(8 * i + 10 * j), q) * a.scale % q);
    a.negoff = ((1ull << 56) / q + 1) * q;
}

static int pointwise_attrs(pmlg_ctx *ctx)
{
    static bool attr_done = false;
    if (!attr_done) {
        const size_t smem_i8 = (size_t)PW_PPC * 8 * 64 * I8_LD;
        const size_t smem_cc2 = 2ull * CC2_STAGE * sizeof(uint32_t);
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_i8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_i8));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_cc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cc2));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_f16_kernel<true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, F16_SMEM));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_f16_kernel<true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, F16_SMEM));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_f16_kernel<false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, F16_SMEM));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_f16_kernel<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, F16_SMEM));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_f16_kernel<true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, F16_SMEM));
        PMLG_CUDA_TRY(cudaFuncSetAttribute(pw_f16_kernel<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, F16_SMEM));
        attr_done = true;
    }
    return PMLG_OK;
}

// one launch of the pointwise products in the given (concrete) form
static int pointwise_run(pmlg_ctx *ctx, const PwArgs &a, int f, cudaStream_t st)
{
    const int64_t grid = (a.npts + PW_PPC - 1) / PW_PPC;
    if (grid > 0x7fffffffll) return PMLG_EUNSUP;
    if (f == PMLG_FORM_INT8_TC) {
        const size_t smem_i8 = (size_t)PW_PPC * 8 * 64 * I8_LD;
        prof_begin(ctx, "pointwise_int8_tc", st);
        pw_i8_kernel<<<(unsigned)grid, PW_THREADS, smem_i8, st>>>(a);
    } else if (f == PMLG_FORM_F16_TC) {
        PwArgs b = a;
        b.err = ctx->d_err;
        // point pairs share 8 aligned bytes in the point-tiled layout
        const bool tile = a.pt_tile == kPtTile && a.s_e == kPtTile && a.s_p == 1 && (a.npts & 1) == 0 &&
                          ((uintptr_t)a.A.base & 7) == 0 && ((uintptr_t)a.B.base & 7) == 0 &&
                          ((uintptr_t)a.C & 7) == 0 && (a.A.s_tile & 1) == 0 && (a.B.s_tile & 1) == 0 &&
                          (a.s_tile_c & 1) == 0;
        int mx = a.r > a.k ? a.r : a.k;
        mx = mx > a.c ? mx : a.c;
        b.lmt = 3;
        while ((1 << b.lmt) < mx) b.lmt++;
        const int64_t units = (a.npts + (128 >> b.lmt) - 1) / (128 >> b.lmt);
        const int64_t g3 = units < ctx->sm_count ? units : ctx->sm_count;
        prof_begin(ctx, "pointwise_f16_tc", st);
        const bool pack = b.lmt < 6;
        const bool skip = a.r < 64 || a.c < 64;   // some epilogue warps hold no output of a region
        if (tile && pack)
            pw_f16_kernel<true, true, true><<<(unsigned)g3, F16_THREADS, F16_SMEM, st>>>(b);
        else if (tile && skip)
            pw_f16_kernel<true, false, true><<<(unsigned)g3, F16_THREADS, F16_SMEM, st>>>(b);
        else if (tile)
            pw_f16_kernel<true, false, false><<<(unsigned)g3, F16_THREADS, F16_SMEM, st>>>(b);
        else if (pack)
            pw_f16_kernel<false, true, true><<<(unsigned)g3, F16_THREADS, F16_SMEM, st>>>(b);
        else if (skip)
            pw_f16_kernel<false, false, true><<<(unsigned)g3, F16_THREADS, F16_SMEM, st>>>(b);
        else
            pw_f16_kernel<false, false, false><<<(unsigned)g3, F16_THREADS, F16_SMEM, st>>>(b);
    } else {
        const size_t smem_cc2 = 2ull * CC2_STAGE * sizeof(uint32_t);
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

uint64_t tune_key(int r, int k, int c, int64_t npts)
{
    int lp = 0;
    while (lp < 62 && (1ll << lp) < npts) lp++;
    return ((uint64_t)r << 32) | ((uint64_t)k << 24) | ((uint64_t)c << 16) | (uint64_t)lp;
}

// PMLG_FORM_AUTO: the form measured fastest for this shape class (r, k, c and the
// number of points rounded up to a power of two).  The first product of a class runs
// each of the three forms twice on its own data, timed by events on its stream, and
// keeps the fastest; every form writes the same bits, so the output is right whichever
// ran last.  No measurement while the stream is being captured, when the products
// accumulate into C, under per-kernel profiling, or with tuning switched off: the FP16
// form, fastest on every large workload, is taken then.
static int pointwise_auto(pmlg_ctx *ctx, const PwArgs &a, cudaStream_t st)
{
    const uint64_t key = tune_key(a.r, a.k, a.c, a.npts);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) return pointwise_run(ctx, a, it->second, st);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PMLG_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
    if (!ctx->tuning || a.accumulate || ctx->profiling || cs != cudaStreamCaptureStatusNone)
        return pointwise_run(ctx, a, PMLG_FORM_F16_TC, st);
    static const int forms[3] = {PMLG_FORM_CUDA_CORE, PMLG_FORM_INT8_TC, PMLG_FORM_F16_TC};
    cudaEvent_t ev[7] = {};
    int s = PMLG_OK;
    for (int i = 0; i < 7 && s == PMLG_OK; i++)
        if (cudaEventCreate(&ev[i]) != cudaSuccess) s = PMLG_ECUDA;
    if (s == PMLG_OK && cudaEventRecord(ev[0], st) != cudaSuccess) s = PMLG_ECUDA;
    for (int f = 0; f < 3 && s == PMLG_OK; f++) {
        // a first run of each form, then the timed one
        s = pointwise_run(ctx, a, forms[f], st);
        if (s == PMLG_OK && cudaEventRecord(ev[1 + 2 * f], st) != cudaSuccess) s = PMLG_ECUDA;
        if (s == PMLG_OK) s = pointwise_run(ctx, a, forms[f], st);
        if (s == PMLG_OK && cudaEventRecord(ev[2 + 2 * f], st) != cudaSuccess) s = PMLG_ECUDA;
    }
    int best = PMLG_FORM_F16_TC;
    if (s == PMLG_OK && cudaEventSynchronize(ev[6]) == cudaSuccess) {
        float bt = 0.f;
        for (int f = 0; f < 3; f++) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, ev[1 + 2 * f], ev[2 + 2 * f]) != cudaSuccess) continue;
            if (f == 0 || t < bt) { bt = t; best = forms[f]; }
        }
        ctx->tuned[key] = best;
    } else if (s == PMLG_OK) {
        s = PMLG_ECUDA;
    }
    for (int i = 0; i < 7; i++)
        if (ev[i]) cudaEventDestroy(ev[i]);
    if (s == PMLG_ECUDA) set_error(ctx, "pointwise form tuning: an event operation failed");
    return s;
}

int pointwise_launch(pmlg_ctx *ctx, const PwArgs &a, int form, cudaStream_t st)
{
    PMLG_TRY(pointwise_attrs(ctx));
    if (a.npts <= 0) return PMLG_OK;
    if (form == PMLG_FORM_AUTO) return pointwise_auto(ctx, a, st);
    return pointwise_run(ctx, a, form, st);
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
