"""GPU parity tests of the modular dot products and multimodular CRT."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, as_u64, golden, to_dev, vec_from_seed

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", golden("dots"), ids=lambda c: f"p{c['p']}-n{c['n']}-s{c['seed1']}")
def test_dot_golden(ctx, case):
    import pml_gb300
    import torch
    p, n = case["p"], case["n"]
    v1 = vec_from_seed(n, p, case["seed1"])
    v2 = vec_from_seed(n, p, case["seed2"])
    assert pml_gb300.nmod_vec_dot_product(to_dev(v1), to_dev(v2), p, ctx=ctx) == case["dot"]
    if p <= 2 ** 32:
        d1 = torch.from_numpy(v1.astype(np.uint32).view(np.int32)).cuda()
        d2 = torch.from_numpy(v2.astype(np.uint32).view(np.int32)).cuda()
        assert pml_gb300.nmod32_vec_dot_product(d1, d2, p, ctx=ctx) == case["dot"]


@pytest.mark.parametrize("n", [1 << 20, (1 << 24) + 3])
def test_dot_large_and_unreduced(ctx, n):
    """Long vectors, and 64-bit entries not reduced mod p (the 3-limb case of
    nmod_vec_dot_product.c:68-127)."""
    import pml_gb300
    p = P998
    rng = np.random.default_rng(n)
    v1 = rng.integers(0, 2 ** 63, n, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    v2 = rng.integers(0, 2 ** 63, n, dtype=np.uint64)
    assert pml_gb300.nmod_vec_dot_product(to_dev(v1), to_dev(v2), p, ctx=ctx) == oracle.nmod_vec_dot(v1, v2, p)


def test_mdot_and_multi(ctx):
    import pml_gb300
    import torch
    p = 1515531527 if oracle.is_prime(1515531527) else 1515531521
    mat = oracle.rand_vec_u32(37 * 130, p, 5).reshape(37, 130)
    vec = oracle.rand_vec_u32(120, p, 6)
    dm = torch.from_numpy(mat.view(np.int32)).cuda()
    dv = torch.from_numpy(vec.view(np.int32)).cuda()
    out = pml_gb300.nmod32_vec_mdot(dm[:, :].contiguous(), dv, p, ctx=ctx)
    # mdot over the first len = 120 columns with stride 130
    ref = oracle.nmod32_vec_mdot(mat, vec, p)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
    # dot_multi: uv[j] = sum_i u[i] v[i, j]
    q = 2 ** 61 - 1
    u = oracle.rand_vec(500, q, 7)
    v = oracle.rand_vec(500 * 9, q, 8).reshape(500, 9)
    uv = pml_gb300.nmod_vec_dot_product_multi(to_dev(u), to_dev(v), q, ctx=ctx)
    ref = [oracle.nmod_vec_dot(u, np.ascontiguousarray(v[:, j]), q) for j in range(9)]
    assert list(uv.cpu().numpy().view(np.uint64)) == ref


@pytest.mark.parametrize("case", golden("crts"), ids=lambda c: f"np{len(c['primes'])}-p{c['p']}")
def test_crt_golden(ctx, case):
    import pml_gb300
    res = as_u64(case["residues"])
    out = pml_gb300.nmod_multimod_CRT_CRT(to_dev(res), case["primes"], case["p"], ctx=ctx)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), as_u64(case["out"]))


def test_multimod_roundtrip(ctx):
    """reduce -> CRT is the identity mod p for values below the prime product."""
    import pml_gb300
    primes = [659706976665601, 910395627798529, 1086317488242689]
    p = 2 ** 61 - 1
    x = oracle.rand_vec(100000, p, 9)
    res = pml_gb300.nmod_multimod_CRT_reduce(to_dev(x), primes, ctx=ctx)
    assert np.array_equal(res.cpu().numpy().view(np.uint64), oracle.multimod_reduce(x, primes))
    back = pml_gb300.nmod_multimod_CRT_CRT(res, primes, p, ctx=ctx)
    assert np.array_equal(back.cpu().numpy().view(np.uint64), x)


def test_dot_long_rows_unaligned_and_tails(ctx):
    """The streaming dot products on their fast and fallback paths: 16-byte aligned and
    unaligned views, lengths that leave tails after the unrolled loops, rows long
    enough for the block-per-row matrix-vector kernel, all-(p-1) worst cases."""
    import pml_gb300
    import torch
    rng = np.random.default_rng(17)
    p64 = 2 ** 63 - 25
    base = rng.integers(0, p64, 40003, dtype=np.uint64)
    base2 = rng.integers(0, p64, 40003, dtype=np.uint64)
    db, db2 = to_dev(base), to_dev(base2)
    for off, n in [(0, 40003), (1, 40001), (0, 7), (1, 3), (0, 0)]:
        got = pml_gb300.nmod_vec_dot_product(db[off:off + n], db2[off:off + n], p64, ctx=ctx)
        assert got == oracle.nmod_vec_dot(base[off:off + n], base2[off:off + n], p64), (off, n)
    worst = np.full(9999, p64 - 1, dtype=np.uint64)
    assert pml_gb300.nmod_vec_dot_product(to_dev(worst), to_dev(worst), p64, ctx=ctx) == \
        oracle.nmod_vec_dot(worst, worst, p64)
    p32 = 4294967291
    w32 = rng.integers(0, p32, 50003, dtype=np.uint64).astype(np.uint32)
    x32 = rng.integers(0, p32, 50003, dtype=np.uint64).astype(np.uint32)
    dw = torch.from_numpy(w32.view(np.int32)).cuda()
    dx = torch.from_numpy(x32.view(np.int32)).cuda()
    for off, n in [(0, 50003), (1, 50001), (3, 50000), (2, 5)]:
        got = pml_gb300.nmod32_vec_dot_product(dw[off:off + n], dx[off:off + n], p32, ctx=ctx)
        ref = oracle.nmod_vec_dot(w32[off:off + n].astype(np.uint64), x32[off:off + n].astype(np.uint64), p32)
        assert got == ref, (off, n)
    # matrix-vector with rows of 4999 entries (block per row) at stride 5003, and short rows
    for nrows, ln, stride in [(50, 4999, 5003), (33, 8192, 8192), (5, 100, 101)]:
        mat = rng.integers(0, p32, nrows * stride, dtype=np.uint64).astype(np.uint32).reshape(nrows, stride)
        if nrows == 33:
            mat[:] = p32 - 1
        vec = rng.integers(0, p32, ln, dtype=np.uint64).astype(np.uint32)
        if nrows == 33:
            vec[:] = p32 - 1
        dm = torch.from_numpy(mat.view(np.int32)).cuda()
        dv = torch.from_numpy(vec.view(np.int32)).cuda()
        out = pml_gb300.nmod32_vec_mdot(dm, dv, p32, ctx=ctx)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), oracle.nmod32_vec_mdot(mat, vec, p32)), nrows
    # dot_multi with a length that is not a multiple of the eight rows in flight
    q = 2 ** 61 - 1
    u = oracle.rand_vec(1003, q, 18)
    v = oracle.rand_vec(1003 * 37, q, 19).reshape(1003, 37)
    uv = pml_gb300.nmod_vec_dot_product_multi(to_dev(u), to_dev(v), q, ctx=ctx)
    ref = [oracle.nmod_vec_dot(u, np.ascontiguousarray(v[:, j]), q) for j in range(37)]
    assert list(uv.cpu().numpy().view(np.uint64)) == ref


@pytest.mark.parametrize("ln,k,off", [(1003, 36, 0), (64, 2, 0), (777, 40, 1), (5000, 512, 0)])
def test_dot_multi_column_pairs(ctx, ln, k, off):
    """Vector-matrix products with an even number of columns (two columns per thread,
    16-byte loads) and, at an 8-byte offset, the one-column fallback."""
    import pml_gb300
    q = 2 ** 63 - 25
    u = oracle.rand_vec(ln, q, 20 + k)
    flat = oracle.rand_vec(ln * k + off, q, 21 + k)
    v = flat[off:].reshape(ln, k)
    dv = to_dev(flat)[off:].view(ln, k)
    uv = pml_gb300.nmod_vec_dot_product_multi(to_dev(u), dv, q, ctx=ctx)
    ref = [oracle.nmod_vec_dot(u, np.ascontiguousarray(v[:, j]), q) for j in range(k)]
    assert list(uv.cpu().numpy().view(np.uint64)) == ref


@pytest.mark.parametrize("primes,p", [
    ([9223372036854775783, 9223372036854775643, 9223372036854775549, 9223372036854775507], 9223372036854775783),
    ([9223372036854775783, 9223372036854775643, 9223372036854775549], 18446744073709551557),
    ([659706976665601, 910395627798529, 1086317488242689, 1108307720798209], 2 ** 61 - 1),
    ([9223372036854775783], 2),
    ([1000003, 1000033, 1000037, 1000039, 1000081, 1000099], 9223372036854775807)])
def test_multimod_crt_bounds(ctx, primes, p):
    """CRT back mod p with primes just below 2^63 (the largest Barrett remainders and
    Shoup products), p just below and above 2^63 (the 64-bit and the 128-bit kernels),
    six primes, residues all q_j - 1 and random."""
    import pml_gb300
    rng = np.random.default_rng(len(primes) + p % 1000)
    nb = 5000
    res = np.stack([rng.integers(0, q, nb, dtype=np.uint64) for q in primes])
    res[:, 0] = [q - 1 for q in primes]
    res[:, 1] = 0
    out = pml_gb300.nmod_multimod_CRT_CRT(to_dev(res), primes, p, ctx=ctx)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), oracle.multimod_crt(res, primes, p))
