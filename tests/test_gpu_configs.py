"""GPU parity at the benchmark workloads themselves, at full size, bit for bit
against the oracle (the reference's tests compare with FLINT in the same way:
t-mul_geometric.c:40-43, t-pmbasis.c:70-107).  The inputs are the ones
bench.py times, from the same seeds:

- the 64x64 . 64x64 product of length 4096 mod 998244353, every pointwise form
  and the tuned default, on device buffers and through the host-buffer entry
  point;
- the 4096 batched 64x64 matrix products mod 998244353 (uint32), every form;
- pmbasis of the 64x32 matrix at order 8192, zero shift: basis and shifted row
  degree, and appbas * F = 0 mod x^8192 by the GPU product;
- the 256 batched uneven products (half of them modulo 59-bit primes), all
  256 outputs.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import bench
import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
FORMS = [0, 1, 2, 3]   # AUTO (tuned), CUDA_CORE, INT8_TC, F16_TC


def test_config3_full_product_every_form(ctx):
    import pml_gb300
    import torch
    A, B = bench.make_inputs(1)
    ref = oracle.poly_mat_mul_ntt(A, B, P998, nthreads=NT)
    dA, dB = to_dev(A), to_dev(B)
    for form in FORMS:
        ctx.set_form(form)
        C = pml_gb300.nmod_poly_mat_multiply(dA, dB, P998, ctx=ctx)
        torch.cuda.synchronize()
        assert np.array_equal(to_host(C), ref), f"form {form}"
        del C
    ctx.set_form(3)
    Ch = pml_gb300.nmod_poly_mat_multiply(A, B, P998, ctx=ctx)   # host buffers: pmlg_poly_mat_mul_host
    ctx.set_form(0)
    assert np.array_equal(Ch, ref)


def test_config2_all_batches_every_form(ctx):
    import pml_gb300
    import torch
    A, B = bench.pointwise_batch_inputs(11)
    ref = oracle.nmod_mat_mul_batch_u32(A, B, P998, nthreads=NT)
    dA = torch.from_numpy(A.view(np.int32)).cuda()
    dB = torch.from_numpy(B.view(np.int32)).cuda()
    for form in FORMS:
        ctx.set_form(form)
        C = pml_gb300.nmod_mat_mul_batch(dA, dB, P998, ctx=ctx)
        torch.cuda.synchronize()
        assert np.array_equal(C.cpu().numpy().view(np.uint32), ref), f"form {form}"
    ctx.set_form(0)


def test_config4_pmbasis_order_8192(ctx):
    import pml_gb300
    import torch
    F = bench.pmbasis_input(7)
    m, n, order = F.shape[0], F.shape[1], F.shape[2]
    dF = to_dev(F)
    ab, sh = pml_gb300.nmod_poly_mat_pmbasis(dF, order, [0] * m, P998, ctx=ctx)
    torch.cuda.synchronize()
    ref, rsh = oracle.pmbasis(F, order, [0] * m, P998, nthreads=NT)
    assert list(sh) == list(rsh)
    assert np.array_equal(to_host(ab), ref)
    # the approximant property, on the GPU: appbas * F = 0 mod x^order
    R = pml_gb300.nmod_poly_mat_multiply(ab.contiguous(), dF, P998, ctx=ctx)
    torch.cuda.synchronize()
    assert not bool(R[:, :, :order].any().item())


def test_config5_all_instances(ctx):
    import pml_gb300
    import torch
    inst = bench.uneven_instances(5)
    jobs = [(to_dev(A), to_dev(B), p) for A, B, p in inst]
    outs = pml_gb300.nmod_poly_mat_multiply_batch(jobs, ctx=ctx)
    torch.cuda.synchronize()
    for i, ((A, B, p), o) in enumerate(zip(inst, outs)):
        ref = oracle.poly_mat_mul_fast(A, B, p, nthreads=NT)
        assert np.array_equal(to_host(o), ref), f"instance {i}: {A.shape[0]}x{A.shape[0]}, len {A.shape[2]}, p {p}"
