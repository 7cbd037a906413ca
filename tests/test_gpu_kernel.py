"""GPU parity of the left kernel basis (pmlg_kernel_zls through pml_gb300):
the basis, its pivot indices and shifted row degrees equal the oracle's
(kernel.c:232-480 restated) bit for bit, on the shapes and shift families of
the reference's t-kernel.c, with its degenerate inputs (zero matrix, zero
rows, dependent columns, a single row or column)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu


def _gpu_kernel(ctx, F, shift, p, cap=None):
    import pml_gb300
    ker, piv, rdeg = pml_gb300.nmod_poly_mat_kernel(to_dev(F), shift, p, ctx=ctx, cap=cap)
    return to_host(ker), list(piv), list(rdeg)


def _same(ctx, F, shift, p):
    ker, piv, rdeg = _gpu_kernel(ctx, F, shift, p)
    rker, rpiv, rrdeg, nul = oracle.kernel_zls(F, shift, p, nthreads=8)
    assert ker.shape[0] == nul
    assert piv == list(rpiv) and rdeg == list(rrdeg)
    L = max(ker.shape[2], rker.shape[2])
    pad = lambda a: np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)
    assert np.array_equal(pad(ker), pad(rker))
    return ker, piv, rdeg


@pytest.mark.parametrize("dims", [(4, 2, 3), (8, 3, 4), (10, 4, 6), (5, 3, 4), (16, 4, 8), (20, 7, 5),
                                  (7, 6, 3), (9, 9, 2), (2, 5, 3), (32, 12, 10), (48, 16, 6), (64, 20, 4)])
def test_kernel_random(ctx, dims):
    m, n, d = dims
    p = P998
    F = oracle.rand_poly_mat(m, n, d + 1, p, 100 + m + n)
    for shift in ([0] * m, list(range(m)), [(7 * i) % 5 for i in range(m)]):
        _same(ctx, F, shift, p)


def test_kernel_degenerate(ctx):
    p = P998
    m = 6
    ker, piv, rdeg = _same(ctx, np.zeros((m, 3, 4), dtype=np.uint64), [0] * m, p)
    assert len(piv) == m
    F = oracle.rand_poly_mat(m, 3, 5, p, 9)
    F[2] = 0
    F[:, 2] = F[:, 0]
    _same(ctx, F, [0] * m, p)
    _same(ctx, oracle.rand_poly_mat(1, 3, 4, p, 10), [0], p)
    _same(ctx, oracle.rand_poly_mat(5, 1, 4, p, 11), [0] * 5, p)
    _same(ctx, oracle.rand_poly_mat(12, 4, 6, 536870923, 12), [0] * 12, 536870923)


def test_kernel_property_and_small_buffer(ctx):
    """K * F = 0 through the GPU product, and a buffer shorter than the basis is
    reported (PMLG_ELEN with the needed length) and then filled on retry."""
    import pml_gb300
    p = P998
    F = oracle.rand_poly_mat(24, 8, 9, p, 31)
    ker, piv, rdeg = _gpu_kernel(ctx, F, [0] * 24, p, cap=1)
    assert ker.shape[0] == 16
    prod = to_host(pml_gb300.nmod_poly_mat_multiply(to_dev(ker), to_dev(F), p, ctx=ctx))
    assert not prod.any()


def test_kernel_host_path(ctx):
    """The host-buffer entry point (numpy in, numpy out) equals the device one."""
    import pml_gb300
    p = P998
    F = oracle.rand_poly_mat(10, 4, 7, p, 41)
    kh, ph, rh = pml_gb300.nmod_poly_mat_kernel(F, list(range(10)), p, ctx=ctx)
    kd, pd, rd = _gpu_kernel(ctx, F, list(range(10)), p)
    assert np.array_equal(kh, kd) and list(ph) == pd and list(rh) == rd


@pytest.mark.parametrize("dims", [(6, 2, 4), (8, 3, 3), (7, 3, 5), (3, 6, 2), (5, 5, 2), (2, 7, 3), (40, 12, 6),
                                  (12, 40, 5)])
@pytest.mark.parametrize("orient", ["ROW_LOWER", "ROW_UPPER", "COL_UPPER", "COL_LOWER"])
def test_kernel_orientations(ctx, dims, orient):
    """pmlg_kernel in every orientation, default shift and an explicit one, against the
    oracle's nmod_poly_mat_kernel (kernel.c:26-144) bit for bit."""
    import pml_gb300
    r, c, d = dims
    p = P998
    F = oracle.rand_poly_mat(r, c, d + 1, p, r * c + d)
    m = r if orient.startswith("ROW") else c
    for shift in (None, [(5 * i) % 3 for i in range(m)]):
        ker, piv, sh = pml_gb300.nmod_poly_mat_kernel_oriented(to_dev(F), p, orient, shift, ctx=ctx)
        rker, rpiv, rsh, nul = oracle.kernel(F, shift, p, orient)
        ker = to_host(ker)
        assert list(piv) == list(rpiv)
        if shift is not None:
            assert list(sh) == list(rsh)
        L = max(ker.shape[2], rker.shape[2])
        pad = lambda a: np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)
        assert np.array_equal(pad(ker), pad(rker))


@pytest.mark.parametrize("dims", [(6, 2, 4), (8, 3, 3), (5, 5, 2), (1, 3, 4), (16, 4, 6)])
def test_kernel_via_approx(ctx, dims):
    import pml_gb300
    m, n, d = dims
    p = P998
    F = oracle.rand_poly_mat(m, n, d + 1, p, 7 * m + n)
    for shift in ([0] * m, list(range(m))):
        ker, piv, rdeg = pml_gb300.nmod_poly_mat_kernel_via_approx(to_dev(F), shift, p, ctx=ctx)
        rker, rpiv, rrdeg, nul = oracle.kernel_via_approx(F, shift, p)
        ker = to_host(ker)
        assert ker.shape[0] == nul and list(piv) == list(rpiv) and list(rdeg) == list(rrdeg)
        L = max(ker.shape[2], rker.shape[2])
        pad = lambda a: np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)
        assert np.array_equal(pad(ker), pad(rker))
    Z = np.zeros((4, 2, 3), dtype=np.uint64)
    ker, piv, rdeg = pml_gb300.nmod_poly_mat_kernel_via_approx(to_dev(Z), [0] * 4, p, ctx=ctx)
    assert ker.shape[0] == 4 and list(piv) == [0, 1, 2, 3]
