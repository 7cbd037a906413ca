"""A fixed-seed randomized differential sweep of the GPU library against the
oracle: products (every form, moduli from 20 to 62 bits, device and host
buffers), middle products, pmbasis and shift-Popov bases (random shifts, zero
rows), kernel bases in every orientation, and batches of products; then long
products and middle products (transforms of 4096 to 16384 points, moduli up to
2^64 - 59), Dixon lifting and truncated inverses (singular inputs included) and
layout round trips.  Bounded to a fixed number of cases so it runs in seconds."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev, to_host

pytestmark = pytest.mark.gpu

CASES = 140


def _pad(a, L):
    return np.concatenate([a, np.zeros(a.shape[:2] + (L - a.shape[2],), dtype=np.uint64)], axis=2)


def test_random_sweep(ctx):
    import pml_gb300
    rng = np.random.default_rng(2026)
    kinds = ["mul", "mulhost", "mulmid", "pmbasis", "popov", "kernel", "batch"]
    for case in range(CASES):
        kind = kinds[case % len(kinds)]
        pbits = int(rng.integers(20, 63)) if kind in ("mul", "mulhost", "mulmid", "batch") else int(rng.integers(20, 31))
        p = P998 if rng.random() < 0.3 else oracle.rand_prime(pbits, int(rng.integers(1, 10 ** 6)))
        seed = int(rng.integers(1, 10 ** 9))
        info = (case, kind, p, seed)
        if kind in ("mul", "mulhost", "mulmid"):
            r, k, c = (int(x) for x in rng.integers(1, 20, size=3))
            l1, l2 = (int(x) for x in rng.integers(1, 200, size=2))
            A = oracle.rand_poly_mat(r, k, l1, p, seed)
            B = oracle.rand_poly_mat(k, c, l2, p, seed + 1)
            ctx.set_form(int(rng.integers(0, 4)))
            if kind == "mul":
                out = to_host(pml_gb300.nmod_poly_mat_multiply(to_dev(A), to_dev(B), p, ctx=ctx))
                ref = oracle.poly_mat_mul(A, B, p, nthreads=8)
            elif kind == "mulhost":
                out = pml_gb300.nmod_poly_mat_multiply(A, B, p, ctx=ctx)
                ref = oracle.poly_mat_mul(A, B, p, nthreads=8)
            else:
                nlo = int(rng.integers(0, l1 + l2))
                nhi = nlo + int(rng.integers(1, l1 + l2))
                out = to_host(pml_gb300.nmod_poly_mat_mulmid(to_dev(A), to_dev(B), nlo, nhi, p, ctx=ctx))
                ref = oracle.poly_mat_mulmid(A, B, nlo, nhi, p, nthreads=8)[0]
            ctx.set_form(0)
            assert out.shape == ref.shape and np.array_equal(out, ref), info
        elif kind in ("pmbasis", "popov"):
            m = int(rng.integers(1, 65))
            n = int(rng.integers(1, min(m, 32) + 1))
            order = int(rng.integers(1, 120))
            F = oracle.rand_poly_mat(m, n, int(rng.integers(1, order + 5)), p, seed)
            if rng.random() < 0.3:
                F[int(rng.integers(0, m))] = 0
            sh = [int(x) for x in rng.integers(0, order, size=m)] if rng.random() < 0.5 else [0] * m
            fn = pml_gb300.nmod_poly_mat_pmbasis if kind == "pmbasis" else pml_gb300.nmod_poly_mat_popov_pmbasis
            ofn = oracle.pmbasis if kind == "pmbasis" else oracle.popov_pmbasis
            ab, s2 = fn(to_dev(F), order, sh, p, ctx=ctx)
            ref, rs = ofn(F, order, sh, p, nthreads=8)
            ab = to_host(ab)
            L = max(ab.shape[2], ref.shape[2])
            assert list(s2) == list(rs) and np.array_equal(_pad(ab, L), _pad(ref, L)), info
        elif kind == "kernel":
            r, c = (int(x) for x in rng.integers(1, 33, size=2))
            F = oracle.rand_poly_mat(r, c, int(rng.integers(1, 8)), p, seed)
            orient = ["ROW_LOWER", "ROW_UPPER", "COL_UPPER", "COL_LOWER"][case % 4]
            ker, piv, _ = pml_gb300.nmod_poly_mat_kernel_oriented(to_dev(F), p, orient, None, ctx=ctx)
            rk, rp, _, nul = oracle.kernel(F, None, p, orient)
            ker = to_host(ker)
            L = max(ker.shape[2], rk.shape[2])
            assert list(piv) == list(rp) and np.array_equal(_pad(ker, L), _pad(rk, L)), info
        else:
            jobs, refs = [], []
            for j in range(int(rng.integers(1, 8))):
                m = int(rng.integers(1, 20))
                ln = int(rng.integers(1, 200))
                A = oracle.rand_poly_mat(m, m, ln, p, seed + 2 * j)
                B = oracle.rand_poly_mat(m, m, ln, p, seed + 2 * j + 1)
                jobs.append((to_dev(A), to_dev(B), p))
                refs.append(oracle.poly_mat_mul(A, B, p, nthreads=8))
            outs = pml_gb300.nmod_poly_mat_multiply_batch(jobs, ctx=ctx)
            assert all(np.array_equal(to_host(o), r) for o, r in zip(outs, refs)), info


WIDE_CASES = 60


def test_random_sweep_wide(ctx):
    import pml_gb300
    rng = np.random.default_rng(2027)
    kinds = ["bigmul", "bigmulmid", "dixon", "invtrunc", "layout"]
    for case in range(WIDE_CASES):
        kind = kinds[case % len(kinds)]
        seed = int(rng.integers(1, 10 ** 9))
        if kind in ("bigmul", "bigmulmid"):
            plist = [P998, 2, 1000003, oracle.rand_prime(int(rng.integers(31, 65)), seed), 18446744073709551557]
            p = plist[int(rng.integers(0, len(plist)))]
            r, k, c = (int(x) for x in rng.integers(1, 4, size=3))
            l1, l2 = (int(x) for x in rng.integers(1, 3000, size=2))
            A = oracle.rand_poly_mat(r, k, l1, p, seed)
            B = oracle.rand_poly_mat(k, c, l2, p, seed + 1)
            ctx.set_form(int(rng.integers(0, 4)))
            if kind == "bigmul":
                out = to_host(pml_gb300.nmod_poly_mat_multiply(to_dev(A), to_dev(B), p, ctx=ctx))
                ref = oracle.poly_mat_mul(A, B, p, nthreads=8)
            else:
                nlo = int(rng.integers(0, l1 + l2))
                nhi = nlo + int(rng.integers(1, l1 + l2))
                out = to_host(pml_gb300.nmod_poly_mat_mulmid(to_dev(A), to_dev(B), nlo, nhi, p, ctx=ctx))
                ref = oracle.poly_mat_mulmid(A, B, nlo, nhi, p, nthreads=8)[0]
            ctx.set_form(0)
            assert out.shape == ref.shape and np.array_equal(out, ref), (case, kind, p, seed)
        elif kind in ("dixon", "invtrunc"):
            plist = [P998, 536870923, 1000003]
            p = plist[int(rng.integers(0, len(plist)))]
            n = int(rng.integers(1, 33))
            alen = int(rng.integers(1, 40))
            order = int(rng.integers(1, 70))
            A = oracle.rand_poly_mat(n, n, alen, p, seed)
            if rng.random() < 0.15:
                A[:, :, 0] = 0   # A(0) singular
            if kind == "invtrunc":
                S, inv = pml_gb300.nmod_poly_mat_inv_trunc(to_dev(A), order, p, ctx=ctx)
                rS, rinv = oracle.inv_trunc(A, order, p, nthreads=8)
                assert bool(inv) == bool(rinv), (case, kind, seed)
                if rinv:
                    assert np.array_equal(to_host(S)[:, :, :order], rS[:, :, :order]), (case, kind, seed)
            else:
                m = int(rng.integers(1, 33))
                blen = int(rng.integers(1, 200))
                sigma = int(rng.integers(0, 400))
                B = oracle.rand_poly_mat(n, m, blen, p, seed + 1)
                X, ok = pml_gb300.nmod_poly_mat_dixon(to_dev(A), to_dev(B), order, sigma, p, ctx=ctx)
                rX, rok = oracle.dixon(A, B, order, sigma, p, nthreads=8)
                assert bool(ok) == bool(rok), (case, kind, seed)
                if rok:
                    assert np.array_equal(to_host(X), rX), (case, kind, seed)
        else:
            r, c = (int(x) for x in rng.integers(1, 70, size=2))
            ln = int(rng.integers(1, 3000))
            order = int(rng.integers(0, 3500))
            P = rng.integers(0, 2 ** 63, size=(r, c, ln), dtype=np.uint64)
            if rng.random() < 0.5:
                P[:, :, int(rng.integers(0, ln)):] = 0
            M, L = pml_gb300.nmod_mat_poly_set_trunc_from_poly_mat(to_dev(P), order, ctx=ctx)
            rM, rL = oracle.poly_mat_to_mat_poly(P, order)
            back = pml_gb300.nmod_poly_mat_set_trunc_from_mat_poly(M, order, ctx=ctx)
            assert L == rL and np.array_equal(to_host(M), rM), (case, kind, seed)
            assert np.array_equal(to_host(back), oracle.mat_poly_to_poly_mat(rM, order)), (case, kind, seed)
