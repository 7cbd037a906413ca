"""CPU tests: pin the oracle against the golden fixtures (independent Python
big-integer restatements, tests/golden/make_golden.py) and check the
oracle's own algorithmic invariants.  No GPU involved."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, as_u64, golden, pm_from_seed, vec_from_seed


@pytest.mark.parametrize("case", golden("products"), ids=lambda c: f"p{c['p']}-{c['r']}x{c['k']}x{c['c']}-{c['len1']}-{c['len2']}")
def test_products_golden(case):
    p = case["p"]
    A = pm_from_seed(case["r"], case["k"], case["len1"], p, case["seedA"])
    B = pm_from_seed(case["k"], case["c"], case["len2"], p, case["seedB"])
    C = oracle.poly_mat_mul(A, B, p)
    assert np.array_equal(C, as_u64(case["C"]))


@pytest.mark.parametrize("case", golden("mulmids"), ids=lambda c: f"p{c['p']}-{c['len1']}-{c['len2']}-{c['nlo']}-{c['nhi']}")
def test_mulmid_golden(case):
    p = case["p"]
    A = pm_from_seed(case["r"], case["k"], case["len1"], p, case["seedA"])
    B = pm_from_seed(case["k"], case["c"], case["len2"], p, case["seedB"])
    res, n = oracle.poly_mat_mulmid(A, B, case["nlo"], case["nhi"], p)
    assert n == case["len"]
    assert np.array_equal(res, as_u64(case["res"]))


@pytest.mark.parametrize("case", golden("dots"), ids=lambda c: f"p{c['p']}-n{c['n']}-s{c['seed1']}")
def test_dots_golden(case):
    p, n = case["p"], case["n"]
    v1 = vec_from_seed(n, p, case["seed1"])
    v2 = vec_from_seed(n, p, case["seed2"])
    assert oracle.nmod_vec_dot(v1, v2, p) == case["dot"]
    if p <= 2 ** 32:
        assert oracle.nmod32_vec_dot(v1.astype(np.uint32), v2.astype(np.uint32), p) == case["dot"]
    exact = sum(int(a) * int(b) for a, b in zip(v1, v2))
    assert oracle.integer_dot(v1, v2) == exact


@pytest.mark.parametrize("case", golden("matmuls"), ids=lambda c: f"p{c['p']}-{c['r']}-s{c['seedA']}")
def test_matmul_golden(case):
    p, r, k, c = case["p"], case["r"], case["k"], case["c"]
    A = vec_from_seed(r * k, p, case["seedA"]).reshape(r, k)
    B = vec_from_seed(k * c, p, case["seedB"]).reshape(k, c)
    if case["seedA"] == -1:
        B = A
    assert np.array_equal(oracle.nmod_mat_mul(A, B, p), as_u64(case["C"]))
    Cb = oracle.nmod_mat_mul_batch_u32(A[None].astype(np.uint32), B[None].astype(np.uint32), p)
    assert np.array_equal(Cb[0].astype(np.uint64), as_u64(case["C"]))


@pytest.mark.parametrize("case", golden("crts"), ids=lambda c: f"np{len(c['primes'])}-p{c['p']}")
def test_crt_golden(case):
    res = as_u64(case["residues"])
    out = oracle.multimod_crt(res, case["primes"], case["p"])
    assert np.array_equal(out, as_u64(case["out"]))


@pytest.mark.parametrize("case", golden("nullspaces"), ids=lambda c: f"p{c['p']}-{c['m']}x{c['n']}")
def test_nullspace_golden(case):
    nul, X, perm = oracle.left_nullspace_compact(as_u64(case["A"]), case["p"])
    assert nul == case["nullity"]
    assert list(perm) == case["perm"]
    if nul:
        assert np.array_equal(X, as_u64(case["X"]))


def _approx_input(case):
    if "F" in case:
        return as_u64(case["F"])
    return pm_from_seed(case["m"], case["n"], case["flen"], case["p"], case["seed"])


@pytest.mark.parametrize("case", golden("approx"), ids=lambda c: f"p{c['p']}-{c['m']}x{c['n']}-o{c['order']}-{c['family']}")
def test_approx_golden(case):
    p, order = case["p"], case["order"]
    F = _approx_input(case)
    ref = as_u64(case["appbas"])
    for fn in (lambda: oracle.mbasis(F, order, case["shift_in"], p),
               lambda: oracle.pmbasis(F, order, case["shift_in"], p, thres=1),
               lambda: oracle.pmbasis(F, order, case["shift_in"], p, thres=3),
               lambda: oracle.pmbasis(F, order, case["shift_in"], p, thres=32)):
        ab, sh = fn()
        assert list(sh) == case["shift_out"]
        assert ab.shape == ref.shape
        assert np.array_equal(ab, ref)
    assert oracle.is_approximant_basis(ref, F, order, case["shift_in"], p) == 0


def test_ntt_port_matches_schoolbook():
    p = P998
    A = oracle.rand_poly_mat(5, 4, 37, p, 1)
    B = oracle.rand_poly_mat(4, 6, 50, p, 2)
    assert np.array_equal(oracle.poly_mat_mul_ntt(A, B, p, nthreads=2), oracle.poly_mat_mul(A, B, p))


@pytest.mark.parametrize("p", [2, 1000003, P998, 549755813911, 562949953421381, 576460752303423619,
                               (1 << 63) - 25, (1 << 64) - 59])
def test_crt_product_matches_schoolbook(p):
    """The multi-prime product (NTT products modulo up to six primes below 2^30,
    Garner's CRT) equals the schoolbook definition for moduli up to 2^64, with
    all-(p-1) entries (the largest integer coefficients) and random ones."""
    for (r, k, c, l1, l2, seed) in [(3, 4, 5, 17, 33, 1), (2, 7, 2, 60, 9, 2), (4, 3, 4, 33, 33, -1)]:
        A = pm_from_seed(r, k, l1, p, seed)
        B = pm_from_seed(k, c, l2, p, seed if seed == -1 else seed + 10)
        assert np.array_equal(oracle.poly_mat_mul_crt(A, B, p, nthreads=2), oracle.poly_mat_mul(A, B, p))


@pytest.mark.parametrize("seed", range(6))
def test_pmbasis_reference_style(seed):
    """t-pmbasis.c:449-489 style: random prime, dims, order; verified basis,
    independent of the leaf threshold."""
    rng = np.random.default_rng(seed)
    bits = int(rng.integers(2, 30))
    p = oracle.rand_prime(bits, seed) if bits > 2 else 3
    m, n = int(rng.integers(1, 8)), int(rng.integers(1, 8))
    order = int(rng.integers(0, 40))
    flen = int(rng.integers(1, 40))
    F = oracle.rand_poly_mat(m, n, flen, p, 100 + seed)
    for shift in ([0] * m, list(range(m)), list(range(m, 0, -1))):
        ab, sh = oracle.pmbasis(F, order, shift, p, thres=4)
        ab2, sh2 = oracle.mbasis(F, order, shift, p)
        assert np.array_equal(ab, ab2) and list(sh) == list(sh2)
        assert oracle.is_approximant_basis(ab, F, order, shift, p) == 0


def test_verifier_rejects_wrong_basis():
    """A mistake planted in an oracle output must be caught by the verifier."""
    p = P998
    F = oracle.rand_poly_mat(4, 2, 16, p, 5)
    ab, _ = oracle.pmbasis(F, 16, [0] * 4, p)
    bad = ab.copy()
    bad[1, 2, 0] = (bad[1, 2, 0] + 1) % p
    assert oracle.is_approximant_basis(bad, F, 16, [0] * 4, p) != 0


def test_find_root_and_primes():
    # nmod_find_root (nmod_find_root.c:21-38) returns the smallest q whose
    # order exceeds n, 0 if there is none
    assert oracle.find_root(4, 5) == 0
    assert oracle.find_root(4, 7) == 3
    assert oracle.is_prime(P998) and not oracle.is_prime(P998 + 2)
    q = oracle.rand_prime(59, 7)
    assert q.bit_length() == 59 and oracle.is_prime(q)


@pytest.mark.parametrize("primes,p", [
    ([9223372036854775783, 9223372036854775643, 9223372036854775549, 9223372036854775507], 9223372036854775783),
    ([9223372036854775783, 9223372036854775643, 9223372036854775549], 18446744073709551557),
    ([1000003, 1000033, 1000037, 1000039, 1000081, 1000099], 9223372036854775807),
    ([9223372036854775783], 2)])
def test_multimod_oracle_against_big_integers(primes, p):
    """The oracle's multimodular reduction and CRT (the checker of the GPU kernels at
    primes just below 2^63 and p on both sides of 2^63) against Python big integers."""
    from math import prod
    rng = np.random.default_rng(len(primes))
    nb = 200
    res = np.stack([rng.integers(0, q, nb, dtype=np.uint64) for q in primes])
    res[:, 0] = [q - 1 for q in primes]
    out = oracle.multimod_crt(res, primes, p)
    M = prod(primes)
    for i in range(nb):
        x = 0
        for j, q in enumerate(primes):
            Mj = M // q
            x += int(res[j, i]) * Mj * pow(Mj, -1, q)
        assert int(out[i]) == (x % M) % p
    x = rng.integers(0, 2 ** 63, nb, dtype=np.uint64)
    red = oracle.multimod_reduce(x, primes)
    assert all(int(red[j, i]) == int(x[i]) % q for j, q in enumerate(primes) for i in range(nb))


def test_dot_oracle_against_big_integers():
    """The oracle's dot products at the largest entries (all p - 1, 64- and 32-bit) against
    Python big integers."""
    for p, n in [(2 ** 63 - 25, 5000), (2 ** 64 - 59, 3000), (4294967291, 7000)]:
        a = np.full(n, p - 1, dtype=np.uint64)
        b = np.random.default_rng(n).integers(0, p, n, dtype=np.uint64)
        assert oracle.nmod_vec_dot(a, b, p) == sum(int(u) * int(v) for u, v in zip(a, b)) % p


@pytest.mark.parametrize("p", [P998, 2 ** 61 - 1, 18446744073709551557])
def test_dot_multi_oracle_against_big_integers(p):
    """The oracle's vector-matrix dot product (every column an exact sum, one
    reduction) against Python big integers, random and all-(p-1) entries."""
    u = oracle.rand_vec(257, p, 1)
    v = oracle.rand_vec(257 * 9, p, 2).reshape(257, 9)
    ref = [sum(int(a) * int(b) for a, b in zip(u, v[:, j])) % p for j in range(9)]
    assert list(oracle.nmod_vec_dot_multi(u, v, p, nthreads=2)) == ref
    u = np.full(4097, p - 1, dtype=np.uint64)
    v = np.full((4097, 3), p - 1, dtype=np.uint64)
    assert list(oracle.nmod_vec_dot_multi(u, v, p)) == [4097 * (p - 1) * (p - 1) % p] * 3
