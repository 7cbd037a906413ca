"""GPU truncated inverse and Dixon lifting (pmlg_inv_trunc, pmlg_dixon) against
the oracle (nmod_poly_mat_dixon.c restated), bit for bit, with the singular case
reported, and the defining property A X = B mod x^sigma at a larger size."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,alen,order", [(1, 3, 5), (3, 4, 10), (8, 6, 33), (16, 5, 64), (32, 4, 40)])
def test_inv_trunc(ctx, n, alen, order):
    import pml_gb300
    p = P998
    A = oracle.rand_poly_mat(n, n, alen, p, n + alen)
    S, ok = pml_gb300.nmod_poly_mat_inv_trunc(to_dev(A), order, p, ctx=ctx)
    rS, rok = oracle.inv_trunc(A, order, p, nthreads=8)
    assert ok and rok and np.array_equal(to_host(S), rS)


@pytest.mark.parametrize("n,m,alen,blen,order,sigma", [(3, 2, 4, 5, 10, 35), (5, 1, 2, 3, 4, 30),
                                                        (8, 3, 6, 6, 33, 104), (4, 4, 3, 9, 7, 7), (2, 2, 2, 2, 5, 0),
                                                        (16, 8, 5, 5, 32, 200)])
def test_dixon(ctx, n, m, alen, blen, order, sigma):
    import pml_gb300
    p = P998
    A = oracle.rand_poly_mat(n, n, alen, p, 3 * n)
    B = oracle.rand_poly_mat(n, m, blen, p, 5 * m)
    X, ok = pml_gb300.nmod_poly_mat_dixon(to_dev(A), to_dev(B), order, sigma, p, ctx=ctx)
    rX, rok = oracle.dixon(A, B, order, sigma, p, nthreads=8)
    assert ok and rok and np.array_equal(to_host(X), rX)


@pytest.mark.parametrize("p", [1000003, 1073741789, 998244353])
@pytest.mark.parametrize("n,m,alen,blen,order,sigma", [(4, 3, 5, 7, 16, 100), (6, 2, 9, 40, 12, 130),
                                                        (3, 5, 2, 3, 1, 20)])
def test_dixon_primes_and_lengths(ctx, p, n, m, alen, blen, order, sigma):
    """Moduli that take one NTT prime or CRT over several, a right-hand side longer
    than the digits (the residue shrinks over the first steps, so the middle product's
    transform size changes and the kept evaluations of the inverse are made again), and
    digits of one coefficient: bit-exact against the oracle."""
    import pml_gb300
    A = oracle.rand_poly_mat(n, n, alen, p, 7 * n + alen)
    B = oracle.rand_poly_mat(n, m, blen, p, 11 * m + blen)
    X, ok = pml_gb300.nmod_poly_mat_dixon(to_dev(A), to_dev(B), order, sigma, p, ctx=ctx)
    rX, rok = oracle.dixon(A, B, order, sigma, p, nthreads=8)
    assert ok == rok
    if rok:
        assert np.array_equal(to_host(X), rX)


def test_singular_and_property(ctx):
    import pml_gb300
    p = P998
    A = oracle.rand_poly_mat(4, 4, 3, p, 1)
    A[:, :, 0] = 0
    assert not pml_gb300.nmod_poly_mat_inv_trunc(to_dev(A), 8, p, ctx=ctx)[1]
    assert not pml_gb300.nmod_poly_mat_dixon(to_dev(A), to_dev(oracle.rand_poly_mat(4, 1, 3, p, 2)), 4, 8, p,
                                             ctx=ctx)[1]
    # A X = B mod x^sigma through the GPU product at 32 x 32, sigma = 1000
    A = oracle.rand_poly_mat(32, 32, 8, p, 5)
    B = oracle.rand_poly_mat(32, 4, 8, p, 6)
    X, ok = pml_gb300.nmod_poly_mat_dixon(to_dev(A), to_dev(B), 64, 1000, p, ctx=ctx)
    assert ok
    AX = to_host(pml_gb300.nmod_poly_mat_multiply(to_dev(A), X, p, ctx=ctx))[:, :, :1000]
    Bs = np.zeros((32, 4, 1000), dtype=np.uint64)
    Bs[:, :, :8] = B
    assert np.array_equal(AX, Bs)
