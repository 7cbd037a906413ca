"""GPU layout conversions between entry-major and coefficient-major polynomial
matrices (nmod_mat_poly_set_from.c:31-52, nmod_poly_mat_utils.c:185-210)
against the oracle: truncation, zero padding, the normalised length, empty and
ragged shapes, and a full-size round trip (64x64, length 4096)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(3, 4, 10), (1, 1, 1), (7, 5, 33), (64, 64, 100), (2, 3, 0), (0, 4, 5)])
@pytest.mark.parametrize("order", [0, 1, 7, 64, 1000])
def test_layout_round_trip(ctx, shape, order):
    import pml_gb300
    r, c, ln = shape
    P = oracle.rand_poly_mat(r, c, ln, P998, 7 + r + ln) if r * c * ln else np.zeros(shape, dtype=np.uint64)
    if ln > 3:
        P[:, :, ln - 3:] = 0            # trailing zero coefficients: the normalised length is shorter
    M, L = pml_gb300.nmod_mat_poly_set_trunc_from_poly_mat(to_dev(P), order, ctx=ctx)
    ref, rL = oracle.poly_mat_to_mat_poly(P, order)
    assert np.array_equal(to_host(M), ref) and L == rL
    K = min(order, ln)
    if r * c:
        Q = pml_gb300.nmod_poly_mat_set_trunc_from_mat_poly(to_dev(ref), order, ctx=ctx)
        assert np.array_equal(to_host(Q), oracle.mat_poly_to_poly_mat(ref, order))
        assert np.array_equal(to_host(Q), P[:, :, :K])


def test_layout_padding_and_full_size(ctx):
    import pml_gb300
    import torch
    P = oracle.rand_poly_mat(64, 64, 4096, P998, 3)
    dP = to_dev(P)
    out = torch.full((4100, 64, 64), -1, dtype=torch.int64, device=dP.device)   # wider than the length
    M, L = pml_gb300.nmod_mat_poly_set_trunc_from_poly_mat(dP, 5000, ctx=ctx, out=out)
    assert L == 4096
    Mh = to_host(M)
    assert np.array_equal(Mh[:4096], np.transpose(P, (2, 0, 1))) and not Mh[4096:].any()
    back = torch.full((64, 64, 4099), -1, dtype=torch.int64, device=dP.device)
    Q = pml_gb300.nmod_poly_mat_set_trunc_from_mat_poly(M[:4096].contiguous(), 4096, ctx=ctx, out=back)
    Qh = to_host(Q)
    assert np.array_equal(Qh[:, :, :4096], P) and not Qh[:, :, 4096:].any()
