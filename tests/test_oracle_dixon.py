"""The oracle's truncated inverse and Dixon lifting (nmod_poly_mat_dixon.c
restated) against their defining properties: S A = A S = I mod x^order,
A X = B mod x^sigma, and the report of a singular A(0).  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998


def _eye(n, L):
    I = np.zeros((n, n, L), dtype=np.uint64)
    I[np.arange(n), np.arange(n), 0] = 1
    return I


@pytest.mark.parametrize("n,alen,order", [(1, 3, 5), (3, 4, 10), (5, 2, 17), (8, 6, 33), (12, 3, 20)])
def test_oracle_inv_trunc(n, alen, order):
    p = P998
    A = oracle.rand_poly_mat(n, n, alen, p, n + alen)
    S, ok = oracle.inv_trunc(A, order, p)
    assert ok
    assert np.array_equal(oracle.poly_mat_mul(S, A, p)[:, :, :order], _eye(n, order))
    assert np.array_equal(oracle.poly_mat_mul(A, S, p)[:, :, :order], _eye(n, order))
    assert not S[:, :, order:].any()


@pytest.mark.parametrize("n,m,alen,blen,order,sigma", [(3, 2, 4, 5, 10, 35), (5, 1, 2, 3, 4, 30),
                                                        (8, 3, 6, 6, 33, 104), (4, 4, 3, 9, 7, 7), (2, 2, 2, 2, 5, 0)])
def test_oracle_dixon(n, m, alen, blen, order, sigma):
    p = P998
    A = oracle.rand_poly_mat(n, n, alen, p, 3 * n)
    B = oracle.rand_poly_mat(n, m, blen, p, 5 * m)
    X, ok = oracle.dixon(A, B, order, sigma, p)
    assert ok
    AX = oracle.poly_mat_mul(A, X, p)[:, :, :sigma]
    Bs = np.zeros((n, m, sigma), dtype=np.uint64)
    Bs[:, :, :min(blen, sigma)] = B[:, :, :min(blen, sigma)]
    assert np.array_equal(AX, Bs)


def test_oracle_singular():
    p = P998
    A = oracle.rand_poly_mat(4, 4, 3, p, 1)
    A[:, :, 0] = 0
    assert not oracle.inv_trunc(A, 8, p)[1]
    assert not oracle.dixon(A, oracle.rand_poly_mat(4, 1, 3, p, 2), 4, 8, p)[1]
