"""GPU parity tests of the modular dot products and multimodular CRT."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, as_u64, golden, to_dev, vec_from_seed

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", golden("dots"), ids=lambda c: f"p{c['p']}-n{c['n']}-s{c['seed1']}")
def test_dot_golden(ctx, case):
    import pml_gb300
    import torch
    p, n = case["p"], case["n"]
    v1 = vec_from_seed(n, p, case["seed1"])
    v2 = vec_from_seed(n, p, case["seed2"])
    assert pml_gb300.nmod_vec_dot_product(to_dev(v1), to_dev(v2), p, ctx=ctx) == case["dot"]
    if p <= 2 ** 32:
        d1 = torch.from_numpy(v1.astype(np.uint32).view(np.int32)).cuda()
        d2 = torch.from_numpy(v2.astype(np.uint32).view(np.int32)).cuda()
        assert pml_gb300.nmod32_vec_dot_product(d1, d2, p, ctx=ctx) == case["dot"]


@pytest.mark.parametrize("n", [1 << 20, (1 << 24) + 3])
def test_dot_large_and_unreduced(ctx, n):
    """Long vectors, and 64-bit entries not reduced mod p (the 3-limb case of
    nmod_vec_dot_product.c:68-127)."""
    import pml_gb300
    p = P998
    rng = np.random.default_rng(n)
    v1 = rng.integers(0, 2 ** 63, n, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    v2 = rng.integers(0, 2 ** 63, n, dtype=np.uint64)
    assert pml_gb300.nmod_vec_dot_product(to_dev(v1), to_dev(v2), p, ctx=ctx) == oracle.nmod_vec_dot(v1, v2, p)


def test_mdot_and_multi(ctx):
    import pml_gb300
    import torch
    p = 1515531527 if oracle.is_prime(1515531527) else 1515531521
    mat = oracle.rand_vec_u32(37 * 130, p, 5).reshape(37, 130)
    vec = oracle.rand_vec_u32(120, p, 6)
    dm = torch.from_numpy(mat.view(np.int32)).cuda()
    dv = torch.from_numpy(vec.view(np.int32)).cuda()
    out = pml_gb300.nmod32_vec_mdot(dm[:, :].contiguous(), dv, p, ctx=ctx)
    # mdot over the first len = 120 columns with stride 130
    ref = oracle.nmod32_vec_mdot(mat, vec, p)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
    # dot_multi: uv[j] = sum_i u[i] v[i, j]
    q = 2 ** 61 - 1
    u = oracle.rand_vec(500, q, 7)
    v = oracle.rand_vec(500 * 9, q, 8).reshape(500, 9)
    uv = pml_gb300.nmod_vec_dot_product_multi(to_dev(u), to_dev(v), q, ctx=ctx)
    ref = [oracle.nmod_vec_dot(u, np.ascontiguousarray(v[:, j]), q) for j in range(9)]
    assert list(uv.cpu().numpy().view(np.uint64)) == ref


@pytest.mark.parametrize("case", golden("crts"), ids=lambda c: f"np{len(c['primes'])}-p{c['p']}")
def test_crt_golden(ctx, case):
    import pml_gb300
    res = as_u64(case["residues"])
    out = pml_gb300.nmod_multimod_CRT_CRT(to_dev(res), case["primes"], case["p"], ctx=ctx)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), as_u64(case["out"]))


def test_multimod_roundtrip(ctx):
    """reduce -> CRT is the identity mod p for values below the prime product."""
    import pml_gb300
    primes = [659706976665601, 910395627798529, 1086317488242689]
    p = 2 ** 61 - 1
    x = oracle.rand_vec(100000, p, 9)
    res = pml_gb300.nmod_multimod_CRT_reduce(to_dev(x), primes, ctx=ctx)
    assert np.array_equal(res.cpu().numpy().view(np.uint64), oracle.multimod_reduce(x, primes))
    back = pml_gb300.nmod_multimod_CRT_CRT(res, primes, p, ctx=ctx)
    assert np.array_equal(back.cpu().numpy().view(np.uint64), x)
