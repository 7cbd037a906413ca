"""Failure detection and error reporting on the GPU.

Every device-side wait of the kernels (mbarrier phases in the tensor-core
pointwise form, published eliminations in the mbasis leaf) is bounded.  A wait
that gives up sets the context's device error word and the kernel returns; the
host reads the word (pmlg_ctx_device_status, and before every host-buffer or
pmbasis call returns) and reports PMLG_ETIMEOUT, with the context still
usable.  The test makes a wait run out on an mbarrier phase that nothing
completes (no fault, no trap).  Invalid arguments return status codes where the
reference has unchecked preconditions or aborts (nmod_poly_mat_multiply.h:34,45;
verification.c:217)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu

EINVAL, EBADMOD, ETIMEOUT, EUNSUP = 1, 2, 6, 9


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def test_bounded_wait_reaches_the_host(ctx):
    import pml_gb300
    st = ctx.lib.pmlg_ctx_selftest_timeout(ctx.handle, 2_000_000, _stream())
    assert st == ETIMEOUT
    assert b"bounded device wait" in ctx.lib.pmlg_ctx_last_error(ctx.handle)
    # the word is cleared by the read, and the context still computes exactly
    assert ctx.lib.pmlg_ctx_device_status(ctx.handle, _stream()) == 0
    A = oracle.rand_poly_mat(3, 4, 20, P998, 1)
    B = oracle.rand_poly_mat(4, 2, 17, P998, 2)
    ctx.set_form(pml_gb300.FORM_F16_TC)
    out = to_host(pml_gb300.nmod_poly_mat_multiply(to_dev(A), to_dev(B), P998, ctx=ctx))
    ctx.set_form(0)
    assert np.array_equal(out, oracle.poly_mat_mul(A, B, P998))
    assert ctx.lib.pmlg_ctx_device_status(ctx.handle, _stream()) == 0


def test_selftest_limits(ctx):
    assert ctx.lib.pmlg_ctx_selftest_timeout(ctx.handle, 0, _stream()) == EINVAL
    assert ctx.lib.pmlg_ctx_selftest_timeout(ctx.handle, 2_000_000_000, _stream()) == EINVAL


def test_status_codes_and_recovery(ctx):
    import pml_gb300
    from pml_gb300 import PmlgError
    A = to_dev(oracle.rand_poly_mat(2, 2, 8, P998, 3))
    with pytest.raises(PmlgError) as e:
        pml_gb300.nmod_poly_mat_multiply(A, A, 1, ctx=ctx)
    assert e.value.status == EBADMOD
    F = to_dev(oracle.rand_poly_mat(4, 2, 16, P998, 4))
    with pytest.raises(PmlgError) as e:
        pml_gb300.nmod_poly_mat_pmbasis(F, 16, [0] * 4, P998 - 1, ctx=ctx)   # not a prime
    assert e.value.status == EBADMOD
    Fbig = to_dev(np.zeros((1025, 2, 16), dtype=np.uint64))
    with pytest.raises(PmlgError) as e:
        pml_gb300.nmod_poly_mat_pmbasis(Fbig, 16, [0] * 1025, P998, ctx=ctx)    # m > 1024
    assert e.value.status == EUNSUP
    with pytest.raises(PmlgError) as e:
        pml_gb300.nmod_poly_mat_mulmid(A, A, -1, 4, P998, ctx=ctx)
    assert e.value.status == EINVAL
    # nothing was left behind on the device, and a correct call follows
    assert ctx.lib.pmlg_ctx_device_status(ctx.handle, _stream()) == 0
    ab, sh = pml_gb300.nmod_poly_mat_pmbasis(F, 16, [0] * 4, P998, ctx=ctx)
    ref, rsh = oracle.pmbasis(to_host(F), 16, [0] * 4, P998)
    assert list(sh) == list(rsh) and np.array_equal(to_host(ab), ref)


def test_follow_on_status_codes(ctx):
    """Limits and moduli of the kernel-basis, Popov, truncated-inverse, Dixon and
    layout entry points come back as status codes; the context keeps working."""
    import ctypes as C
    import torch
    L = ctx.lib
    st = _stream()
    i64, nul, ic = C.c_int64(0), C.c_int64(0), C.c_int(0)
    sh = (C.c_int64 * 1025)()
    piv = (C.c_int64 * 1025)()
    P = torch.zeros((65, 2, 4), dtype=torch.int64, device="cuda")
    K = torch.zeros((65, 65, 8), dtype=torch.int64, device="cuda")
    # kernel basis: m > 1024 (refused before any device access), a composite modulus
    assert L.pmlg_kernel_zls(ctx.handle, K.data_ptr(), 8, C.byref(i64), piv, sh, P.data_ptr(), 1025, 2, 4, P998,
                             C.byref(nul), st) == EUNSUP
    assert L.pmlg_kernel_zls(ctx.handle, K.data_ptr(), 8, C.byref(i64), piv, sh, P.data_ptr(), 4, 2, 4, P998 - 1,
                             C.byref(nul), st) == EBADMOD
    # truncated inverse and Dixon: n > 512; Dixon output shorter than ceil(sigma / order) * order
    assert L.pmlg_inv_trunc(ctx.handle, K.data_ptr(), P.data_ptr(), 513, 1, 4, P998, C.byref(ic), st) == EUNSUP
    assert L.pmlg_dixon(ctx.handle, K.data_ptr(), 7, P.data_ptr(), P.data_ptr(), 2, 1, 1, 1, 4, 8, P998,
                        C.byref(ic), st) == EINVAL
    # Popov basis: a capacity below order + 1; layout: an output shorter than the truncation
    assert L.pmlg_popov_pmbasis(ctx.handle, K.data_ptr(), 4, sh, P.data_ptr(), 4, 2, 4, 4, P998, None,
                                st) == EINVAL
    assert L.pmlg_poly_mat_to_mat_poly(ctx.handle, K.data_ptr(), 3, P.data_ptr(), 4, 2, 4, 4, 4, None,
                                       st) == EINVAL
    assert ctx.lib.pmlg_ctx_device_status(ctx.handle, st) == 0
