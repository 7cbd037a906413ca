"""GPU shifted Popov approximant bases (pmlg_popov_pmbasis) against the oracle
(popov_pmbasis, mat_lzz_pX_pmbasis.cpp:1527-1557 restated): the basis and its
shifted row degree bit for bit, the Popov form and the approximant-basis
properties, and the uniqueness of the Popov basis across leaf orders."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu


def _pad(a, L):
    return np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)


@pytest.mark.parametrize("dims", [(4, 2, 12), (6, 3, 20), (8, 2, 33), (10, 4, 40), (5, 1, 17), (32, 16, 96),
                                  (64, 32, 128)])
def test_popov_pmbasis(ctx, dims):
    import pml_gb300
    m, n, order = dims
    p = P998
    F = oracle.rand_poly_mat(m, n, order, p, 7 * m + n)
    for shift in ([0] * m, list(range(m)), [order * (m - i) for i in range(m)], [(3 * i) % 4 for i in range(m)]):
        ab, sh = pml_gb300.nmod_poly_mat_popov_pmbasis(to_dev(F), order, shift, p, ctx=ctx)
        ab = to_host(ab)
        ref, rsh = oracle.popov_pmbasis(F, order, shift, p, nthreads=8)
        L = max(ab.shape[2], ref.shape[2])
        assert list(sh) == list(rsh)
        assert np.array_equal(_pad(ab, L), _pad(ref, L))
        if m <= 10:
            assert oracle.is_popov(ab, shift)
            assert oracle.is_approximant_basis(ab, F, order, shift, p) == 0


def test_popov_unique_across_leaf_orders(ctx):
    """The s-Popov approximant basis is unique: every leaf order gives the same bits."""
    import pml_gb300
    p = P998
    F = oracle.rand_poly_mat(8, 3, 48, p, 5)
    shift = [5, 0, 2, 9, 1, 1, 0, 3]
    outs = []
    for leaf in (1, 4, 32):
        ctx.set_leaf_order(leaf)
        ab, sh = pml_gb300.nmod_poly_mat_popov_pmbasis(to_dev(F), 48, shift, p, ctx=ctx)
        outs.append((to_host(ab), list(sh)))
    ctx.set_leaf_order(0)
    L = max(o[0].shape[2] for o in outs)
    assert all(np.array_equal(_pad(o[0], L), _pad(outs[0][0], L)) and o[1] == outs[0][1] for o in outs)
