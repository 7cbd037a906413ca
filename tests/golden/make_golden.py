"""Generates the golden fixtures of tests/golden/ with pure-Python big integers.

These restatements are independent of the C oracle (oracle/pmlg_oracle.c) and
of the GPU library; they pin both.  What each fixture follows in the reference
(flint-extras, vneiger/pml):

* products / middle products: the unique answer mod p of
  nmod_poly_mat_multiply (nmod_poly_mat_extra/mul.c:19) and
  nmod_poly_mat_mulmid (mulmid.c:499-541, including the nhi clamp to
  len1+len2-1 computed from the actual lengths); cases after
  test/t-mul_geometric.c:24-51 and test/t-mulmid.c:20-86 (random primes of
  several sizes, small dimensions, the transposed-product constraints);
* dot products: nmod32_vec/test/t-dot.c:19-138 including its worst case with
  every entry equal to p-1, and nmod_vec_extra/test/t-integer_dot_product.c;
* matrix products: nmod_mat_extra/test/t-mul_2dot.c:24-52 (against plain
  nmod_mat_mul), with the all-(p-1) worst case;
* CRT: nmod_extra/test/t-multimod_CRT_{reduce,CRT}.c with the reference's
  fixed primes (nmod_extra.h:65-68);
* left nullspace (compact form of left_nullspace.c:42-102) from an
  independent Python RREF;
* mbasis / pmbasis: a direct Python restatement of nmod_mat_poly_mbasis.c:116-378
  (pmbasis output is independent of the leaf order, so mbasis at the full order
  gives the pmbasis answer), with the shift families of
  nmod_poly_mat_extra/test/t-pmbasis.c:70-107, each basis also checked by a
  Python restatement of nmod_poly_mat_is_approximant_basis (verification.c:21-116).

Run: python tests/golden/make_golden.py   (writes tests/golden/*.json)
"""
from __future__ import annotations

import json
import random
from pathlib import Path

HERE = Path(__file__).resolve().parent

# ---------------------------------------------------------------------------
# generator (identical stream to the oracle: SplitMix64 + rejection)
# ---------------------------------------------------------------------------
M64 = (1 << 64) - 1


def splitmix64(state):
    state[0] = (state[0] + 0x9E3779B97F4A7C15) & M64
    z = state[0]
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def rand_vec(n, p, seed):
    st = [seed & M64]
    lim = M64 - ((M64 % p + 1) % p)
    out = []
    while len(out) < n:
        x = splitmix64(st)
        if x <= lim:
            out.append(x % p)
    return out


def rand_pm(r, c, length, p, seed):
    v = rand_vec(r * c * length, p, seed)
    return [[v[(i * c + j) * length:(i * c + j + 1) * length] for j in range(c)] for i in range(r)]


def is_prime(n):
    if n < 2:
        return False
    small = [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37]
    for s in small:
        if n % s == 0:
            return n == s
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in small:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def rand_prime(bits, rng):
    while True:
        x = rng.getrandbits(bits) | (1 << (bits - 1)) | 1
        if is_prime(x):
            return x


# ---------------------------------------------------------------------------
# polynomial matrix arithmetic
# ---------------------------------------------------------------------------

def max_length(P):
    L = 0
    for row in P:
        for e in row:
            l = len(e)
            while l > L and e[l - 1] == 0:
                l -= 1
            L = max(L, l)
    return L


def pm_mul(A, B, p):
    r, k, c = len(A), len(B), len(B[0])
    l1, l2 = len(A[0][0]), len(B[0][0])
    n = l1 + l2 - 1 if l1 and l2 else 0
    out = [[[0] * n for _ in range(c)] for _ in range(r)]
    for i in range(r):
        for j in range(c):
            acc = [0] * n
            for l in range(k):
                a, b = A[i][l], B[l][j]
                for d1, x in enumerate(a):
                    if x:
                        for d2, y in enumerate(b):
                            acc[d1 + d2] += x * y
            out[i][j] = [v % p for v in acc]
    return out


def pm_mulmid(A, B, nlo, nhi, p):
    cap = max(nhi - nlo, 0)
    r, c = len(A), len(B[0])
    L1, L2 = max_length(A), max_length(B)
    hi = min(nhi, L1 + L2 - 1)
    res = [[[0] * cap for _ in range(c)] for _ in range(r)]
    if L1 == 0 or L2 == 0 or nlo >= hi:
        return res, 0
    full = pm_mul(A, B, p)
    for i in range(r):
        for j in range(c):
            for t in range(nlo, hi):
                res[i][j][t - nlo] = full[i][j][t] if t < len(full[i][j]) else 0
    return res, hi - nlo


def mat_mul(A, B, p):
    return [[sum(A[i][l] * B[l][j] for l in range(len(B))) % p for j in range(len(B[0]))] for i in range(len(A))]


def rref(M, p):
    """reduced row echelon form over GF(p); returns (R, pivot columns)"""
    M = [row[:] for row in M]
    rows, cols = len(M), (len(M[0]) if M else 0)
    piv, r = [], 0
    for c in range(cols):
        if r == rows:
            break
        pr = next((i for i in range(r, rows) if M[i][c] % p), None)
        if pr is None:
            continue
        M[r], M[pr] = M[pr], M[r]
        inv = pow(M[r][c], p - 2, p)
        M[r] = [x * inv % p for x in M[r]]
        for i in range(rows):
            if i != r and M[i][c]:
                f = M[i][c]
                M[i] = [(x - f * y) % p for x, y in zip(M[i], M[r])]
        piv.append(c)
        r += 1
    return M, piv


def left_nullspace_compact(A, p):
    m, n = len(A), len(A[0])
    At = [[A[i][j] for i in range(m)] for j in range(n)]
    R, piv = rref(At, p)
    rank = len(piv)
    nonpiv = [c for c in range(m) if c not in piv]
    if rank == m:
        return 0, [], list(range(m))
    X = [[(-R[b][f]) % p for b in range(rank)] for f in nonpiv]
    return m - rank, X, piv + nonpiv


def mbasis(F, order, shift, p):
    """nmod_mat_poly_mbasis (nmod_mat_poly_mbasis.c:116-378) on lists.
    F[i][j] list of coefficients; returns (appbas [m][m] coefficient lists of
    length alen, shift out)."""
    m, n = len(F), len(F[0])
    shift = list(shift)
    Fc = [[[(F[i][j][d] if d < len(F[i][j]) else 0) for j in range(n)] for i in range(m)] for d in range(order)]
    ab = [[[1 if i == j else 0 for j in range(m)] for i in range(m)]]  # ab[d][i][j]
    if all(F[i][j][d] == 0 for i in range(m) for j in range(n) for d in range(min(order, len(F[i][j])))):
        return to_entries(ab, m), shift
    for ord_ in range(order):
        res = [[0] * n for _ in range(m)]
        for t in range(0, min(ord_ + 1, len(ab))):
            if ord_ - t < order:
                pr = mat_mul(ab[t], Fc[ord_ - t], p)
                res = [[(x + y) % p for x, y in zip(r1, r2)] for r1, r2 in zip(res, pr)]
        perm = sorted(range(m), key=lambda i: (shift[i], i))
        resp = [res[perm[i]] for i in range(m)]
        nullity, X, piv = left_nullspace_compact(resp, p)
        rank = m - nullity
        if nullity == 0:
            k = order - ord_
            ab = [[[0] * m for _ in range(m)] for _ in range(k)] + ab
            shift = [s + k for s in shift]
            break
        if nullity < m:
            piv = [perm[x] for x in piv]
            for i in range(rank):
                shift[piv[i]] += 1
            ab = [[M[piv[i]] for i in range(m)] for M in ab]
            for M in ab:
                upd = mat_mul(X, M[:rank], p)
                for i in range(nullity):
                    M[rank + i] = [(x + y) % p for x, y in zip(M[rank + i], upd[i])]
            if any(ab[-1][i][j] for i in range(rank) for j in range(m)):
                ab.append([[0] * m for _ in range(m)])
            for d in range(len(ab) - 1, 0, -1):
                for i in range(rank):
                    ab[d][i] = ab[d - 1][i][:]
            for i in range(rank):
                ab[0][i] = [0] * m
            inv = [0] * m
            for i, x in enumerate(piv):
                inv[x] = i
            ab = [[M[inv[i]] for i in range(m)] for M in ab]
    return to_entries(ab, m), shift


def to_entries(ab, m):
    L = len(ab)
    out = [[[ab[d][i][j] for d in range(L)] for j in range(m)] for i in range(m)]
    # normalise to the max length
    ml = max_length(out)
    return [[e[:max(ml, 1)] for e in row] for row in out]


def poly_deg(a):
    d = len(a) - 1
    while d >= 0 and a[d] == 0:
        d -= 1
    return d


def is_approximant_basis(ab, F, order, shift, p):
    m, n = len(F), len(F[0])
    # ordered weak Popov, ROW_LOWER
    prev = -1
    for i in range(m):
        best, pj = None, -1
        for j in range(m):
            d = poly_deg(ab[i][j])
            if d >= 0 and (best is None or d + shift[j] >= best):
                best, pj = d + shift[j], j
        if pj < 0 or pj <= prev:
            return False
        prev = pj
    res = pm_mul(ab, F, p)
    for i in range(m):
        for j in range(n):
            if any(res[i][j][t] for t in range(min(order, len(res[i][j])))):
                return False
    CP = [[(ab[i][j][0] if ab[i][j] else 0) for j in range(m)]
          + [(res[i][j][order] if order < len(res[i][j]) else 0) for j in range(n)] for i in range(m)]
    _, piv = rref(CP, p)
    return len(piv) == m


# ---------------------------------------------------------------------------
# fixtures
# ---------------------------------------------------------------------------

def main():
    rng = random.Random(20260101)
    P998 = 998244353
    primes = [P998, 2, 3, 521, 524309, 536870923, rand_prime(40, rng), rand_prime(59, rng), rand_prime(63, rng)]

    products = []
    for idx, p in enumerate(primes):
        for shape in [(1, 1, 1, 1, 1), (2, 3, 4, 5, 7), (3, 2, 3, 9, 4), (4, 4, 4, 12, 12)]:
            r, k, c, l1, l2 = shape
            seed = 1000 * idx + l1 * 7 + l2
            A = rand_pm(r, k, l1, p, seed)
            B = rand_pm(k, c, l2, p, seed + 1)
            products.append({"p": p, "r": r, "k": k, "c": c, "len1": l1, "len2": l2, "seedA": seed,
                             "seedB": seed + 1, "C": pm_mul(A, B, p)})
    # worst case: every coefficient p-1
    for p in [P998, primes[7]]:
        r, k, c, l1, l2 = 3, 5, 2, 6, 6
        A = [[[p - 1] * l1 for _ in range(k)] for _ in range(r)]
        B = [[[p - 1] * l2 for _ in range(c)] for _ in range(k)]
        products.append({"p": p, "r": r, "k": k, "c": c, "len1": l1, "len2": l2, "seedA": -1, "seedB": -1,
                         "C": pm_mul(A, B, p)})
    # x^k identities: A = x^3 * I, B random -> C = x^3 * B
    p = P998
    B = rand_pm(3, 3, 5, p, 77)
    A = [[[0, 0, 0, 1] if i == j else [0, 0, 0, 0] for j in range(3)] for i in range(3)]
    C = pm_mul(A, B, p)
    assert all(C[i][j][3:8] == B[i][j] and C[i][j][:3] == [0, 0, 0] for i in range(3) for j in range(3))

    mulmids = []
    for idx, p in enumerate([P998, 536870923, primes[7]]):
        for (r, k, c, l1, l2, nlo, nhi) in [(2, 3, 2, 5, 9, 4, 11), (3, 3, 2, 4, 16, 6, 12),
                                            (2, 2, 3, 16, 4, 8, 14), (2, 2, 2, 6, 6, 3, 40),
                                            (1, 2, 1, 3, 3, 9, 12), (3, 2, 3, 10, 10, 0, 5)]:
            seed = 5000 + 100 * idx + nlo
            A = rand_pm(r, k, l1, p, seed)
            B = rand_pm(k, c, l2, p, seed + 1)
            res, n = pm_mulmid(A, B, nlo, nhi, p)
            mulmids.append({"p": p, "r": r, "k": k, "c": c, "len1": l1, "len2": l2, "nlo": nlo, "nhi": nhi,
                            "seedA": seed, "seedB": seed + 1, "res": res, "len": n})

    dots = []
    for p in [P998, 1515531527 if is_prime(1515531527) else 1515531521, primes[7], primes[8], 2 ** 64 - 59]:
        for n in [0, 1, 7, 8, 9, 1000]:
            v1 = rand_vec(n, p, 11 + n)
            v2 = rand_vec(n, p, 13 + n)
            dots.append({"p": p, "n": n, "seed1": 11 + n, "seed2": 13 + n,
                         "dot": sum(a * b for a, b in zip(v1, v2)) % p})
        # all entries p-1 (t-dot.c, i == 0)
        n = 4097
        dots.append({"p": p, "n": n, "seed1": -1, "seed2": -1, "dot": (n * (p - 1) * (p - 1)) % p})

    matmuls = []
    for p in [P998, 536870923, 7]:
        for (r, k, c) in [(1, 1, 1), (3, 4, 5), (16, 16, 16), (64, 64, 64)]:
            A = rand_vec(r * k, p, r * 31 + c)
            B = rand_vec(k * c, p, r * 37 + c)
            Am = [A[i * k:(i + 1) * k] for i in range(r)]
            Bm = [B[i * c:(i + 1) * c] for i in range(k)]
            matmuls.append({"p": p, "r": r, "k": k, "c": c, "seedA": r * 31 + c, "seedB": r * 37 + c,
                            "C": mat_mul(Am, Bm, p)})
        r = k = c = 64
        Am = [[p - 1] * k for _ in range(r)]
        matmuls.append({"p": p, "r": r, "k": k, "c": c, "seedA": -1, "seedB": -1, "C": mat_mul(Am, Am, p)})

    crt_primes = [659706976665601, 910395627798529, 1086317488242689, 1108307720798209]
    crts = []
    for np_ in [1, 2, 3, 4]:
        pr = crt_primes[:np_]
        Q = 1
        for q in pr:
            Q *= q
        for p in [P998, primes[7], 2 ** 64 - 59]:
            xs = [rng.randrange(Q) for _ in range(6)] + [0, Q - 1]
            res = [[x % q for x in xs] for q in pr]
            crts.append({"primes": pr, "p": p, "residues": res, "out": [x % p for x in xs]})

    nullspaces = []
    for p in [P998, 3, 524309]:
        for (m, n, rank) in [(5, 3, 3), (6, 4, 2), (4, 4, 4), (7, 2, 0), (8, 3, 1), (6, 6, 5)]:
            # matrix of given rank: product of random m x rank and rank x n
            U = [rand_vec(rank, p, 100 + i) for i in range(m)]
            V = [rand_vec(n, p, 200 + i) for i in range(rank)]
            A = [[sum(U[i][t] * V[t][j] for t in range(rank)) % p for j in range(n)] for i in range(m)] \
                if rank else [[0] * n for _ in range(m)]
            nul, X, perm = left_nullspace_compact(A, p)
            nullspaces.append({"p": p, "m": m, "n": n, "A": A, "nullity": nul, "X": X, "perm": perm})

    approx = []

    def shift_families(m, order, rng):
        fam = {"uniform": [0] * m, "increasing": list(range(m)), "decreasing": list(range(m, 0, -1))}
        sh = list(range(m))
        rng.shuffle(sh)
        fam["shuffle"] = sh
        fam["hermite"] = [order * i for i in range(m)]
        fam["rhermite"] = [order * (m - i) for i in range(m)]
        fam["plateau"] = [0] * (m // 2) + [order] * (m - m // 2)
        fam["rplateau"] = [order] * (m // 2) + [0] * (m - m // 2)
        return fam

    for (p, m, n, order, flen) in [(P998, 4, 2, 12, 12), (P998, 3, 1, 9, 9), (536870923, 5, 3, 10, 8),
                                   (3, 4, 2, 8, 8), (2, 3, 2, 7, 7), (P998, 2, 3, 6, 6),
                                   (524309, 6, 3, 16, 16)]:
        for fname, shift in shift_families(m, order, rng).items():
            seed = 9000 + m * 13 + n + order
            F = rand_pm(m, n, flen, p, seed)
            ab, sh = mbasis(F, order, shift, p)
            assert is_approximant_basis(ab, F, order, shift, p), (p, m, n, order, fname)
            approx.append({"p": p, "m": m, "n": n, "order": order, "flen": flen, "seed": seed, "family": fname,
                           "shift_in": shift, "shift_out": sh, "appbas": ab})
    # word-size primes of the reference's testing collection (40, 50 and 60 bits,
    # testing_collection.h:16-20), a random 64-bit prime, and more than 64 rows
    big = [(549755813911, 4, 2, 12, 12), (562949953421381, 5, 3, 10, 8), (576460752303423619, 3, 2, 9, 9),
           (rand_prime(64, rng), 4, 3, 8, 8), (P998, 66, 2, 4, 4), (576460752303423619, 67, 3, 3, 3)]
    for (p, m, n, order, flen) in big:
        for fname, shift in shift_families(m, order, rng).items():
            seed = 9500 + m * 13 + n + order
            F = rand_pm(m, n, flen, p, seed)
            ab, sh = mbasis(F, order, shift, p)
            assert is_approximant_basis(ab, F, order, shift, p), (p, m, n, order, fname)
            approx.append({"p": p, "m": m, "n": n, "order": order, "flen": flen, "seed": seed, "family": fname,
                           "shift_in": shift, "shift_out": sh, "appbas": ab})
    # Pade-type input [[f], [-1]]: basis verified by the property check
    p = P998
    f = rand_vec(10, p, 4242)
    F = [[f], [[p - 1] + [0] * 9]]
    ab, sh = mbasis(F, 10, [0, 0], p)
    assert is_approximant_basis(ab, F, 10, [0, 0], p)
    approx.append({"p": p, "m": 2, "n": 1, "order": 10, "flen": 10, "seed": -1, "family": "pade",
                   "F": F, "shift_in": [0, 0], "shift_out": sh, "appbas": ab})

    out = {"products": products, "mulmids": mulmids, "dots": dots, "matmuls": matmuls, "crts": crts,
           "nullspaces": nullspaces, "approx": approx}
    for name, data in out.items():
        (HERE / f"{name}.json").write_text(json.dumps(data, separators=(",", ":")))
        print(name, len(data))


if __name__ == "__main__":
    main()
