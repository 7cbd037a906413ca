"""GPU parity tests of the approximant bases (pmlg_pmbasis / pmlg_mbasis through
pml_gb300): bit-exact basis and shifted row degree against the golden
fixtures and the oracle, with the reference's shift families and property
check (nmod_poly_mat_extra/test/t-pmbasis.c)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, as_u64, golden, pm_from_seed, to_dev, to_host

pytestmark = pytest.mark.gpu


def _pm(ctx, F, order, shift, p, fn="pmbasis"):
    import pml_gb300
    import torch
    f = pml_gb300.nmod_poly_mat_pmbasis if fn == "pmbasis" else pml_gb300.nmod_poly_mat_mbasis
    ab, sh = f(to_dev(F), order, shift, p, ctx=ctx)
    torch.cuda.synchronize()
    return to_host(ab), list(sh)


@pytest.mark.parametrize("case", golden("approx"), ids=lambda c: f"p{c['p']}-{c['m']}x{c['n']}-o{c['order']}-{c['family']}")
@pytest.mark.parametrize("leaf", [1, 4, 32])
def test_pmbasis_golden(ctx, case, leaf):
    p, order = case["p"], case["order"]
    F = as_u64(case["F"]) if "F" in case else pm_from_seed(case["m"], case["n"], case["flen"], p, case["seed"])
    ctx.set_leaf_order(leaf)
    ab, sh = _pm(ctx, F, order, case["shift_in"], p)
    ctx.set_leaf_order(0)
    assert sh == case["shift_out"]
    assert np.array_equal(ab, as_u64(case["appbas"]))


@pytest.mark.parametrize("form", [1, 2, 3])
@pytest.mark.parametrize("dims", [(4, 2, 64, 64), (6, 3, 100, 80), (8, 4, 129, 129), (16, 8, 256, 256),
                                  (5, 7, 40, 40), (1, 1, 30, 30), (10, 1, 50, 20)])
def test_pmbasis_random(ctx, dims, form):
    m, n, order, flen = dims
    p = P998
    F = oracle.rand_poly_mat(m, n, flen, p, 1000 + m + order)
    ctx.set_form(form)
    for shift in ([0] * m, list(range(m)), [order * (m - i) for i in range(m)]):
        ab, sh = _pm(ctx, F, order, shift, p)
        ref, rsh = oracle.pmbasis(F, order, shift, p, nthreads=8)
        assert sh == list(rsh)
        assert np.array_equal(ab, ref)
    ctx.set_form(0)


def test_mbasis_entry(ctx):
    p = 536870923
    F = oracle.rand_poly_mat(6, 3, 24, p, 77)
    ab, sh = _pm(ctx, F, 24, [0] * 6, p, fn="mbasis")
    ref, rsh = oracle.mbasis(F, 24, [0] * 6, p)
    assert sh == list(rsh) and np.array_equal(ab, ref)


def test_pmbasis_rank_deficient_and_zero(ctx):
    """Zero input (identity basis, shift unchanged), and an input whose columns
    are dependent (rank-deficient residuals, testing_collection.h:117-207)."""
    p = P998
    Z = np.zeros((4, 2, 10), dtype=np.uint64)
    ab, sh = _pm(ctx, Z, 10, [1, 2, 3, 4], p)
    assert sh == [1, 2, 3, 4]
    assert np.array_equal(ab[:, :, 0], np.eye(4, dtype=np.uint64)) and not ab[:, :, 1:].any()
    F = oracle.rand_poly_mat(5, 1, 40, p, 3)
    F2 = np.concatenate([F, F, F], axis=1)   # three equal columns
    ab, sh = _pm(ctx, F2, 40, [0] * 5, p)
    ref, rsh = oracle.pmbasis(F2, 40, [0] * 5, p)
    assert sh == list(rsh) and np.array_equal(ab, ref)
    assert oracle.is_approximant_basis(ab, F2, 40, [0] * 5, p) == 0


def test_pmbasis_config4_scaled(ctx):
    """64x32 at order 1024 (the bench shape at a size the oracle finishes
    quickly): bit-exact against the oracle, and verified."""
    p = P998
    F = oracle.rand_poly_mat(64, 32, 1024, p, 4)
    ab, sh = _pm(ctx, F, 1024, [0] * 64, p)
    ref, rsh = oracle.pmbasis(F, 1024, [0] * 64, p, nthreads=16)
    assert sh == list(rsh)
    assert np.array_equal(ab, ref)


def test_pmbasis_cluster_nonpivot_columns(ctx):
    """64x32 inputs whose eliminations meet columns without a pivot before the
    rank is full (zero and repeated rows of F, repeated columns): the cluster
    leaf's look-ahead publication and its rebuilt pivot entries, bit-exact
    against the oracle."""
    p = P998
    F = oracle.rand_poly_mat(64, 32, 96, p, 11)
    F[3] = 0
    F[40] = 0
    F[17] = F[5]
    F[:, 9] = F[:, 2]
    F[:, 30] = (3 * F[:, 1]) % p
    for shift in ([0] * 64, [(7 * i) % 13 for i in range(64)]):
        ab, sh = _pm(ctx, F, 96, shift, p)
        ref, rsh = oracle.pmbasis(F, 96, shift, p, nthreads=8)
        assert sh == list(rsh)
        assert np.array_equal(ab, ref)


@pytest.mark.parametrize("dims", [(64, 4, 64), (48, 20, 80), (33, 31, 40), (64, 1, 48), (8, 32, 40),
                                  (64, 32, 64), (17, 9, 70)])
def test_pmbasis_cluster_shapes(ctx, dims):
    """Shapes at and inside the cluster leaf's limits (m <= 64, n <= 32): large
    nullity (several non-pivot row groups per warp when the eliminator forms the
    next residual coefficient), slices whose widths are not multiples of 4 (the
    word-wise update), n = 1, and m < n (nullity 0: appbas times a power of x),
    each with a zero, an increasing and a hermite-like shift."""
    m, n, order = dims
    p = P998
    F = oracle.rand_poly_mat(m, n, order, p, 500 + m + n)
    for shift in ([0] * m, list(range(m)), [order * (m - i) for i in range(m)]):
        ab, sh = _pm(ctx, F, order, shift, p)
        ref, rsh = oracle.pmbasis(F, order, shift, p, nthreads=8)
        assert sh == list(rsh)
        assert np.array_equal(ab, ref)
