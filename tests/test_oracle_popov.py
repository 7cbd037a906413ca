"""The oracle's shifted Popov approximant basis against its defining
properties: Popov form (diagonal monic pivots of strictly largest degree in
their columns), approximant basis of the input at the order (the reference's
verifier, verification.c:21-116), and the same shifted row degree as
pmbasis.  CPU only."""
from __future__ import annotations

import pytest

import oracle
from conftest import P998


@pytest.mark.parametrize("dims", [(4, 2, 12), (6, 3, 20), (8, 2, 33), (10, 4, 40), (5, 1, 17)])
def test_oracle_popov(dims):
    m, n, order = dims
    p = P998
    F = oracle.rand_poly_mat(m, n, order, p, m + order)
    for shift in ([0] * m, list(range(m)), [order * (m - i) for i in range(m)], [(3 * i) % 4 for i in range(m)]):
        P, rd = oracle.popov_pmbasis(F, order, shift, p)
        _, rr = oracle.pmbasis(F, order, shift, p)
        assert oracle.is_popov(P, shift)
        assert oracle.is_approximant_basis(P, F, order, shift, p) == 0
        assert list(rd) == list(rr)
