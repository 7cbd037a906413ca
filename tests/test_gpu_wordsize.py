"""GPU parity of the approximant bases and their callers for word-size primes
(30 to 64 bits, the 64-bit leaf) and for more than 64 rows or columns,
bit for bit against the oracle:

- pmbasis on random inputs drawn as t-pmbasis.c:470-478 draws them (a random
  prime of 2 to 64 bits, dimensions 1..10, order and length below 150), with
  the shift families of t-pmbasis.c:70-107;
- pmbasis at the reference's 40-, 50- and 60-bit primes
  (testing_collection.h:16-20) at the benchmark's 64x32 shape;
- pmbasis with 65 to 100 rows, modulo an NTT prime and a 60-bit prime;
- kernel bases, shift-Popov bases, truncated inverses and Dixon lifting
  modulo word-size primes.
"""
from __future__ import annotations

import random

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu

P40, P50, P60 = 549755813911, 562949953421381, 576460752303423619


def _families(m, order, rng):
    sh = list(range(m))
    rng.shuffle(sh)
    return {"uniform": [0] * m, "increasing": list(range(m)), "decreasing": list(range(m, 0, -1)),
            "shuffle": sh, "hermite": [order * i for i in range(m)], "rhermite": [order * (m - i) for i in range(m)],
            "plateau": [0] * (m // 2) + [order] * (m - m // 2), "rplateau": [order] * (m // 2) + [0] * (m - m // 2)}


def _pm(ctx, F, order, shift, p):
    import pml_gb300
    import torch
    ab, sh = pml_gb300.nmod_poly_mat_pmbasis(to_dev(F), order, shift, p, ctx=ctx)
    torch.cuda.synchronize()
    return to_host(ab), list(sh)


@pytest.mark.parametrize("case", range(24))
def test_pmbasis_random_word_primes(ctx, case):
    rng = random.Random(7000 + case)
    bits = 2 + rng.randrange(63)
    p = oracle.rand_prime(bits, 7100 + case) if bits > 2 else rng.choice([2, 3])
    m, n = 1 + rng.randrange(10), 1 + rng.randrange(10)
    order, flen = rng.randrange(150), rng.randrange(150)
    F = oracle.rand_poly_mat(m, n, max(flen, 1), p, 7200 + case)
    if flen == 0:
        F = F[:, :, :0]
    for fname, shift in _families(m, order, rng).items():
        ab, sh = _pm(ctx, F, order, shift, p)
        ref, rsh = oracle.pmbasis(F, order, shift, p, nthreads=8)
        assert sh == list(rsh), (p, m, n, order, fname)
        assert np.array_equal(ab, ref), (p, m, n, order, fname)


@pytest.mark.parametrize("p", [P40, P50, P60])
def test_pmbasis_reference_primes_64x32(ctx, p):
    F = oracle.rand_poly_mat(64, 32, 128, p, 31)
    for shift in ([0] * 64, [(5 * i) % 17 for i in range(64)]):
        ab, sh = _pm(ctx, F, 128, shift, p)
        ref, rsh = oracle.pmbasis(F, 128, shift, p, nthreads=8)
        assert sh == list(rsh)
        assert np.array_equal(ab, ref)


@pytest.mark.parametrize("dims", [(65, 3, 24), (80, 40, 64), (100, 1, 20), (72, 70, 40)])
@pytest.mark.parametrize("p", [P998, P60])
def test_pmbasis_more_than_64_rows(ctx, dims, p):
    m, n, order = dims
    F = oracle.rand_poly_mat(m, n, order, p, 900 + m + n)
    for shift in ([0] * m, [order * (m - i) for i in range(m)]):
        ab, sh = _pm(ctx, F, order, shift, p)
        ref, rsh = oracle.pmbasis(F, order, shift, p, nthreads=8)
        assert sh == list(rsh)
        assert np.array_equal(ab, ref)


def test_mbasis_word_prime(ctx):
    import pml_gb300
    import torch
    F = oracle.rand_poly_mat(6, 3, 40, P50, 77)
    ab, sh = pml_gb300.nmod_poly_mat_mbasis(to_dev(F), 40, [0] * 6, P50, ctx=ctx)
    torch.cuda.synchronize()
    ref, rsh = oracle.mbasis(F, 40, [0] * 6, P50)
    assert list(sh) == list(rsh) and np.array_equal(to_host(ab), ref)


@pytest.mark.parametrize("p", [P40, P60, (1 << 64) - 59])
@pytest.mark.parametrize("dims", [(8, 3, 4), (16, 4, 8), (70, 20, 3)])
def test_kernel_word_primes(ctx, p, dims):
    import pml_gb300
    m, n, d = dims
    F = oracle.rand_poly_mat(m, n, d + 1, p, 300 + m + n)
    shift = [(3 * i) % 7 for i in range(m)]
    ker, piv, rdeg = pml_gb300.nmod_poly_mat_kernel(to_dev(F), shift, p, ctx=ctx)
    ker = to_host(ker)
    rker, rpiv, rrdeg, nul = oracle.kernel_zls(F, shift, p, nthreads=8)
    assert ker.shape[0] == nul
    assert list(piv) == list(rpiv) and list(rdeg) == list(rrdeg)
    L = max(ker.shape[2], rker.shape[2])
    pad = lambda a: np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)
    assert np.array_equal(pad(ker), pad(rker))


@pytest.mark.parametrize("p", [P50, P60])
def test_popov_word_primes(ctx, p):
    import pml_gb300
    import torch
    F = oracle.rand_poly_mat(6, 3, 24, p, 41)
    for shift in ([0] * 6, [(2 * i) % 5 for i in range(6)]):
        ab, sh = pml_gb300.nmod_poly_mat_popov_pmbasis(to_dev(F), 24, shift, p, ctx=ctx)
        torch.cuda.synchronize()
        ref, rsh = oracle.popov_pmbasis(F, 24, shift, p, nthreads=8)
        assert list(sh) == list(rsh)
        ab = to_host(ab)
        L = max(ab.shape[2], ref.shape[2])
        pad = lambda a: np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)
        assert np.array_equal(pad(ab), pad(ref))


@pytest.mark.parametrize("p", [P40, P60])
def test_inv_trunc_and_dixon_word_primes(ctx, p):
    import pml_gb300
    import torch
    A = oracle.rand_poly_mat(4, 4, 6, p, 51)
    B = oracle.rand_poly_mat(4, 2, 6, p, 52)
    S, ok = pml_gb300.nmod_poly_mat_inv_trunc(to_dev(A), 16, p, ctx=ctx)
    torch.cuda.synchronize()
    rS, rok = oracle.inv_trunc(A, 16, p, nthreads=8)
    assert bool(ok) == bool(rok)
    assert np.array_equal(to_host(S), rS)
    X, ok = pml_gb300.nmod_poly_mat_dixon(to_dev(A), to_dev(B), 8, 40, p, ctx=ctx)
    torch.cuda.synchronize()
    rX, rok = oracle.dixon(A, B, 8, 40, p, nthreads=8)
    assert bool(ok) == bool(rok)
    assert np.array_equal(to_host(X), rX)
