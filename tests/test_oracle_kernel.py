"""The oracle's kernel basis (kernel.c:232-480 restated) against the properties
the reference's t-kernel.c checks through nmod_poly_mat_is_kernel: K * F = 0,
the nullity equals m - rank(F), the rows are in shift-ordered weak Popov form
with increasing pivots, and the returned pivots and shifted row degrees are
those of the rows.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998

P = P998


def _rank_at_point(F, p, a=123457):
    Fa = np.zeros(F.shape[:2], dtype=np.uint64)
    for d in range(F.shape[2] - 1, -1, -1):
        Fa = (Fa.astype(object) * a + F[:, :, d].astype(object)) % p
    return oracle.nmod_mat_rank(np.array(Fa, dtype=np.uint64), p)


def check_kernel(F, shift, p):
    m = F.shape[0]
    ker, piv, rdeg, nul = oracle.kernel_zls(F, shift, p, nthreads=4)
    assert nul == m - _rank_at_point(F, p)
    if nul:
        assert not oracle.poly_mat_mul(ker, F, p).any()
        rd, pv = oracle.row_degrees_and_pivots(ker, shift)
        assert list(pv) == list(piv) and list(rd) == list(rdeg)
        assert all(piv[i] < piv[i + 1] for i in range(nul - 1))
    return ker, piv, rdeg, nul


@pytest.mark.parametrize("dims", [(4, 2, 3), (6, 2, 5), (8, 3, 4), (10, 4, 6), (5, 3, 4), (16, 4, 8),
                                  (12, 5, 3), (20, 7, 5), (3, 1, 4), (7, 6, 3), (9, 9, 2), (2, 5, 3)])
def test_oracle_kernel_random(dims):
    m, n, d = dims
    F = oracle.rand_poly_mat(m, n, d + 1, P, 100 + m + n)
    for shift in ([0] * m, list(range(m)), [(7 * i) % 5 for i in range(m)]):
        check_kernel(F, shift, P)


def test_oracle_kernel_degenerate():
    # zero matrix: identity kernel; zero rows and repeated columns; one row; one column
    m = 6
    Z = np.zeros((m, 3, 4), dtype=np.uint64)
    ker, piv, rdeg, nul = check_kernel(Z, [0] * m, P)
    assert nul == m and list(piv) == list(range(m))
    F = oracle.rand_poly_mat(m, 3, 5, P, 9)
    F[2] = 0
    F[:, 2] = F[:, 0]
    check_kernel(F, [0] * m, P)
    check_kernel(oracle.rand_poly_mat(1, 3, 4, P, 10), [0], P)
    check_kernel(oracle.rand_poly_mat(5, 1, 4, P, 11), [0] * 5, P)
    check_kernel(oracle.rand_poly_mat(5, 1, 4, 7, 12), [0] * 5, 7)


def _pivots_upper(ker, shift):
    """s-row degree and s-pivot (the leftmost column reaching it: ROW_UPPER)."""
    rows, cols, L = ker.shape
    out = []
    for i in range(rows):
        best, bj = None, -1
        for j in range(cols):
            nz = np.nonzero(ker[i, j])[0]
            if len(nz) == 0:
                continue
            v = int(nz[-1]) + int(shift[j])
            if best is None or v > best:
                best, bj = v, j
        out.append(bj)
    return out


@pytest.mark.parametrize("dims", [(6, 2, 4), (8, 3, 3), (7, 3, 5), (3, 6, 2), (5, 5, 2), (2, 7, 3)])
def test_oracle_kernel_orientations(dims):
    """nmod_poly_mat_kernel (kernel.c:26-144): left kernels K F = 0 with pivots on the
    right (ROW_LOWER) or the left (ROW_UPPER), right kernels F K = 0 through the
    transpose, and kernel_via_approx on the same inputs."""
    r, c, d = dims
    p = P
    F = oracle.rand_poly_mat(r, c, d + 1, p, r * c + d)
    for orient in ("ROW_LOWER", "ROW_UPPER"):
        ker, piv, _, nul = oracle.kernel(F, None, p, orient)
        assert nul == r - _rank_at_point(F, p)
        if nul:
            assert not oracle.poly_mat_mul(ker, F, p).any()
            rdeg0 = [max([int(np.nonzero(F[i, j])[0][-1]) for j in range(c) if F[i, j].any()] or [0])
                     for i in range(r)]
            want = oracle.row_degrees_and_pivots(ker, rdeg0)[1] if orient == "ROW_LOWER" else _pivots_upper(ker, rdeg0)
            assert list(piv) == list(want)
    for orient in ("COL_UPPER", "COL_LOWER"):
        ker, piv, _, nul = oracle.kernel(F, None, p, orient)
        assert nul == c - _rank_at_point(F, p)
        if nul:
            assert not oracle.poly_mat_mul(F, ker, p).any()
    ker, piv, rdeg, nul = oracle.kernel_via_approx(F, [0] * r, p)
    assert nul == r - _rank_at_point(F, p)
    if nul:
        assert not oracle.poly_mat_mul(ker, F, p).any()
        rd, pv = oracle.row_degrees_and_pivots(ker, [0] * r)
        assert list(pv) == list(piv) and list(rd) == list(rdeg)
