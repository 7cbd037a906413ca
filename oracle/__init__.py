"""Python view of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

The oracle restates PML's evaluation/interpolation path on the CPU (see
pmlg_oracle.h for what each function follows in the reference and for the
parity status).  It is the checker for the GPU library and the timed CPU
baseline; the product library never imports it.

All polynomial matrices are numpy uint64 arrays of shape (rows, cols, len)
(entry-major, zero padded), matching the C ABI layout.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle

_lib = None
_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_i64p = C.POINTER(C.c_int64)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        sig = {
            "orc_rand_vec": (None, [_u64p, C.c_int64, C.c_uint64, C.c_uint64]),
            "orc_rand_vec_u32": (None, [_u32p, C.c_int64, C.c_uint64, C.c_uint64]),
            "orc_mulmod": (C.c_uint64, [C.c_uint64, C.c_uint64, C.c_uint64]),
            "orc_is_prime": (C.c_int, [C.c_uint64]),
            "orc_rand_prime": (C.c_uint64, [C.c_int, C.c_uint64]),
            "orc_find_root": (C.c_uint64, [C.c_uint64, C.c_uint64]),
            "orc_nmod_mat_mul": (None, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64]),
            "orc_nmod_mat_mul_batch_u32": (None, [_u32p, _u32p, _u32p, C.c_int64, C.c_int64, C.c_int64,
                                                  C.c_int64, C.c_uint64, C.c_int]),
            "orc_nmod_mat_rank": (C.c_int64, [_u64p, C.c_int64, C.c_int64, C.c_uint64]),
            "orc_nmod_mat_rref": (C.c_int64, [_u64p, C.c_int64, C.c_int64, C.c_uint64]),
            "orc_left_nullspace_compact": (C.c_int64, [_u64p, _i64p, _u64p, C.c_int64, C.c_int64, C.c_uint64]),
            "orc_pm_max_length": (C.c_int64, [_u64p, C.c_int64, C.c_int64, C.c_int64]),
            "orc_poly_mat_mul": (None, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                        C.c_int64, C.c_uint64, C.c_int]),
            "orc_poly_mat_mulmid": (C.c_int64, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_int64,
                                                C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_int]),
            "orc_poly_mat_mul_ntt": (C.c_int, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_int64,
                                               C.c_int64, C.c_int64, C.c_uint64, C.c_int]),
            "orc_poly_mat_mul_crt": (C.c_int, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_int64,
                                               C.c_int64, C.c_int64, C.c_uint64, C.c_int]),
            "orc_mbasis": (C.c_int64, [_u64p, _i64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                       C.c_uint64]),
            "orc_pmbasis": (C.c_int64, [_u64p, _i64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                        C.c_uint64, C.c_int64, C.c_int]),
            "orc_is_approximant_basis": (C.c_int, [_u64p, C.c_int64, _u64p, C.c_int64, C.c_int64, C.c_int64,
                                                   C.c_int64, _i64p, C.c_uint64]),
            "orc_nmod_vec_dot": (C.c_uint64, [_u64p, _u64p, C.c_int64, C.c_uint64]),
            "orc_nmod_vec_dot_multi": (None, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_uint64, C.c_int]),
            "orc_nmod32_vec_dot": (C.c_uint32, [_u32p, _u32p, C.c_int64, C.c_uint64]),
            "orc_integer_dot": (None, [_u64p, _u64p, _u64p, C.c_int64]),
            "orc_nmod32_vec_mdot": (None, [_u32p, _u32p, _u32p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64]),
            "orc_multimod_reduce": (None, [_u64p, _u64p, C.c_int64, _u64p, C.c_int]),
            "orc_multimod_crt": (None, [_u64p, _u64p, C.c_int64, _u64p, C.c_int, C.c_uint64]),
            "orc_kernel_zls": (C.c_int64, [C.POINTER(_u64p), _i64p, _i64p, _i64p, _u64p, C.c_int64, C.c_int64,
                                           C.c_int64, C.c_uint64, C.c_int]),
            "orc_free": (None, [C.c_void_p]),
            "orc_kernel_via_approx": (C.c_int64, [C.POINTER(_u64p), _i64p, _i64p, _i64p, _u64p, C.c_int64,
                                                  C.c_int64, C.c_int64, C.c_uint64, C.c_int]),
            "orc_kernel": (C.c_int64, [C.POINTER(_u64p), _i64p, _i64p, _i64p, _u64p, C.c_int64, C.c_int64,
                                       C.c_int64, C.c_uint64, C.c_int, C.c_int]),
            "orc_popov_pmbasis": (C.c_int64, [_u64p, _i64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                              C.c_uint64, C.c_int]),
            "orc_inv_trunc": (C.c_int, [_u64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_int]),
            "orc_dixon": (C.c_int, [_u64p, _u64p, _u64p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                    C.c_int64, C.c_uint64, C.c_int]),
            "orc_poly_mat_to_mat_poly": (C.c_int64, [_u64p, C.c_int64, _u64p, C.c_int64, C.c_int64, C.c_int64,
                                                     C.c_int64, C.c_int64]),
            "orc_mat_poly_to_poly_mat": (None, [_u64p, C.c_int64, _u64p, C.c_int64, C.c_int64, C.c_int64,
                                                C.c_int64]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p64(a):
    return a.ctypes.data_as(_u64p)


def _p32(a):
    return a.ctypes.data_as(_u32p)


def _pi64(a):
    return a.ctypes.data_as(_i64p)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


# ---- generator -------------------------------------------------------------

def rand_vec(n: int, p: int, seed: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint64)
    lib().orc_rand_vec(_p64(out), n, p, seed)
    return out


def rand_vec_u32(n: int, p: int, seed: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().orc_rand_vec_u32(_p32(out), n, p, seed)
    return out


def rand_poly_mat(r: int, c: int, length: int, p: int, seed: int) -> np.ndarray:
    return rand_vec(r * c * length, p, seed).reshape(r, c, length)


def is_prime(n: int) -> bool:
    return bool(lib().orc_is_prime(n))


def rand_prime(bits: int, seed: int) -> int:
    return int(lib().orc_rand_prime(bits, seed))


def find_root(n: int, p: int) -> int:
    return int(lib().orc_find_root(n, p))


# ---- matrices ---------------------------------------------------------------

def nmod_mat_mul(A: np.ndarray, B: np.ndarray, p: int) -> np.ndarray:
    A, B = _c64(A), _c64(B)
    r, k = A.shape
    k2, c = B.shape
    assert k == k2
    out = np.empty((r, c), dtype=np.uint64)
    lib().orc_nmod_mat_mul(_p64(out), _p64(A), _p64(B), r, k, c, p)
    return out


def nmod_mat_mul_batch_u32(A: np.ndarray, B: np.ndarray, p: int, nthreads: int = 1) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.uint32)
    B = np.ascontiguousarray(B, dtype=np.uint32)
    nb, r, k = A.shape
    _, _, c = B.shape
    out = np.empty((nb, r, c), dtype=np.uint32)
    lib().orc_nmod_mat_mul_batch_u32(_p32(out), _p32(A), _p32(B), nb, r, k, c, p, nthreads)
    return out


def nmod_mat_rank(A: np.ndarray, p: int) -> int:
    A = _c64(A)
    return int(lib().orc_nmod_mat_rank(_p64(A), A.shape[0], A.shape[1], p))


def nmod_mat_rref(A: np.ndarray, p: int):
    A = _c64(A).copy()
    rk = lib().orc_nmod_mat_rref(_p64(A), A.shape[0], A.shape[1], p)
    return int(rk), A


def left_nullspace_compact(A: np.ndarray, p: int):
    A = _c64(A)
    m, n = A.shape
    X = np.zeros(m * m + 1, dtype=np.uint64)
    perm = np.zeros(m, dtype=np.int64)
    nullity = int(lib().orc_left_nullspace_compact(_p64(X), _pi64(perm), _p64(A), m, n, p))
    rank = m - nullity
    return nullity, X[: nullity * rank].reshape(nullity, rank), perm


# ---- polynomial matrices ----------------------------------------------------

def pm_max_length(P: np.ndarray) -> int:
    P = _c64(P)
    r, c, L = P.shape
    return int(lib().orc_pm_max_length(_p64(P), r, c, L))


def poly_mat_mul(A: np.ndarray, B: np.ndarray, p: int, nthreads: int = 1) -> np.ndarray:
    A, B = _c64(A), _c64(B)
    r, k, l1 = A.shape
    k2, c, l2 = B.shape
    assert k == k2
    if l1 == 0 or l2 == 0:
        return np.zeros((r, c, 0), dtype=np.uint64)
    out = np.empty((r, c, l1 + l2 - 1), dtype=np.uint64)
    lib().orc_poly_mat_mul(_p64(out), _p64(A), _p64(B), r, k, c, l1, l2, p, nthreads)
    return out


def poly_mat_mul_ntt(A: np.ndarray, B: np.ndarray, p: int, nthreads: int = 1) -> np.ndarray:
    A, B = _c64(A), _c64(B)
    r, k, l1 = A.shape
    _, c, l2 = B.shape
    out = np.empty((r, c, l1 + l2 - 1), dtype=np.uint64)
    rc = lib().orc_poly_mat_mul_ntt(_p64(out), _p64(A), _p64(B), r, k, c, l1, l2, p, nthreads)
    if rc != 0:
        raise ValueError("modulus/length not supported by the NTT port")
    return out


def poly_mat_mul_crt(A: np.ndarray, B: np.ndarray, p: int, nthreads: int = 1) -> np.ndarray:
    """A * B mod any p >= 2 through NTT products modulo up to six primes below 2^30 and
    Garner's CRT (the fast oracle product for moduli that are not NTT primes)."""
    A, B = _c64(A), _c64(B)
    r, k, l1 = A.shape
    _, c, l2 = B.shape
    if l1 == 0 or l2 == 0:
        return np.zeros((r, c, 0), dtype=np.uint64)
    out = np.empty((r, c, l1 + l2 - 1), dtype=np.uint64)
    rc = lib().orc_poly_mat_mul_crt(_p64(out), _p64(A), _p64(B), r, k, c, l1, l2, p, nthreads)
    if rc != 0:
        raise ValueError("product beyond the multi-prime oracle's bound")
    return out


def poly_mat_mul_fast(A: np.ndarray, B: np.ndarray, p: int, nthreads: int = 1) -> np.ndarray:
    """The fastest oracle product for the modulus: the single-prime NTT port when p is an
    NTT prime of the transform length, else the multi-prime product."""
    try:
        return poly_mat_mul_ntt(A, B, p, nthreads=nthreads)
    except ValueError:
        return poly_mat_mul_crt(A, B, p, nthreads=nthreads)


def poly_mat_mulmid(A: np.ndarray, B: np.ndarray, nlo: int, nhi: int, p: int, nthreads: int = 1):
    """Returns (res of capacity nhi-nlo, clamped length)."""
    A, B = _c64(A), _c64(B)
    r, k, l1 = A.shape
    _, c, l2 = B.shape
    cap = max(nhi - nlo, 0)
    out = np.zeros((r, c, cap), dtype=np.uint64)
    if cap == 0:
        return out, 0
    n = lib().orc_poly_mat_mulmid(_p64(out), _p64(A), _p64(B), r, k, c, l1, l2, nlo, nhi, p, nthreads)
    return out, int(n)


def mbasis(F: np.ndarray, order: int, shift, p: int):
    F = _c64(F)
    m, n, flen = F.shape
    sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
    out = np.zeros((m, m, order + 1), dtype=np.uint64)
    L = lib().orc_mbasis(_p64(out), _pi64(sh), _p64(F), m, n, flen, order, p)
    return out[:, :, : max(int(L), 1)], sh


def pmbasis(F: np.ndarray, order: int, shift, p: int, thres: int = 32, nthreads: int = 1):
    F = _c64(F)
    m, n, flen = F.shape
    sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
    out = np.zeros((m, m, order + 1), dtype=np.uint64)
    L = lib().orc_pmbasis(_p64(out), _pi64(sh), _p64(F), m, n, flen, order, p, thres, nthreads)
    return out[:, :, : max(int(L), 1)], sh


def is_approximant_basis(appbas: np.ndarray, F: np.ndarray, order: int, shift_in, p: int) -> int:
    appbas, F = _c64(appbas), _c64(F)
    m, m2, alen = appbas.shape
    _, n, flen = F.shape
    sh = np.ascontiguousarray(shift_in, dtype=np.int64)
    return int(lib().orc_is_approximant_basis(_p64(appbas), alen, _p64(F), flen, m, n, order, _pi64(sh), p))


# ---- kernel basis ----------------------------------------------------------

def kernel_zls(pmat: np.ndarray, shift, p: int, nthreads: int = 1):
    """Left kernel basis by ZLS via approximant bases (kernel.c:232-480).
    Returns (ker, pivind, rdeg, nullity): ker is the (nullity, m, L) array of the
    kernel rows, pivind and rdeg their s-pivot indices and s-row degrees."""
    P = _c64(pmat)
    m, n, plen = P.shape
    sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
    piv = np.zeros(max(m, 1), dtype=np.int64)
    kp = _u64p()
    L = C.c_int64(0)
    nul = int(lib().orc_kernel_zls(C.byref(kp), C.byref(L), _pi64(piv), _pi64(sh), _p64(P), m, n, plen, p,
                                   nthreads))
    flat = np.ctypeslib.as_array(kp, shape=(m * m * L.value,)).copy() if m else np.zeros(0, dtype=np.uint64)
    lib().orc_free(C.cast(kp, C.c_void_p))
    ker = flat.reshape(m, m, L.value)[:nul] if m else np.zeros((0, 0, 1), dtype=np.uint64)
    return ker, piv[:nul].copy(), sh[:nul].copy(), nul


def _take(kp, shape):
    n = int(np.prod(shape))
    flat = np.ctypeslib.as_array(kp, shape=(max(n, 1),)).copy()[:n] if n else np.zeros(0, dtype=np.uint64)
    lib().orc_free(C.cast(kp, C.c_void_p))
    return flat.reshape(shape)


def kernel_via_approx(pmat: np.ndarray, shift, p: int, nthreads: int = 1):
    """nmod_poly_mat_kernel_via_approx (kernel.c:146-227): (ker rows, pivind, rdeg, nullity)."""
    P = _c64(pmat)
    m, n, plen = P.shape
    sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
    piv = np.zeros(max(m, 1), dtype=np.int64)
    kp, L = _u64p(), C.c_int64(0)
    nul = int(lib().orc_kernel_via_approx(C.byref(kp), C.byref(L), _pi64(piv), _pi64(sh), _p64(P), m, n, plen, p,
                                          nthreads))
    ker = _take(kp, (m, m, L.value))[:nul]
    return ker, piv[:nul].copy(), sh[:nul].copy(), nul


ORIENT = {"COL_UPPER": 0, "COL_LOWER": 1, "ROW_UPPER": 2, "ROW_LOWER": 3}


def kernel(pmat: np.ndarray, shift, p: int, orient: str = "ROW_LOWER", nthreads: int = 1):
    """nmod_poly_mat_kernel (kernel.c:26-144), ORD_WEAK_POPOV: (ker, pivind, shift_out,
    nullity).  Left kernels return the (nullity, r, L) rows; right kernels the
    (c, nullity, L) columns.  shift None: the default row / column degrees."""
    P = _c64(pmat)
    r, c, plen = P.shape
    o = ORIENT[orient]
    left = o >= 2
    m = r if left else c
    sh = None if shift is None else np.ascontiguousarray(shift, dtype=np.int64).copy()
    piv = np.zeros(max(m, 1), dtype=np.int64)
    kp, L = _u64p(), C.c_int64(0)
    nul = int(lib().orc_kernel(C.byref(kp), C.byref(L), _pi64(piv), _pi64(sh) if sh is not None else None, _p64(P),
                               r, c, plen, p, o, nthreads))
    K = _take(kp, (m, m, L.value))
    ker = K[:nul] if left else K[:, :nul]
    return ker, piv[:nul].copy(), (sh[:nul].copy() if sh is not None else None), nul


def row_degrees_and_pivots(ker: np.ndarray, shift):
    """s-row degrees and s-pivot indices (the rightmost column reaching the
    s-row degree: ROW_LOWER) of the rows of a polynomial matrix."""
    rows, cols, L = ker.shape
    deg = np.full((rows, cols), -1, dtype=np.int64)
    nz = ker != 0
    for d in range(L):
        deg[nz[:, :, d]] = d
    rdeg, piv = [], []
    for i in range(rows):
        best, bj = None, -1
        for j in range(cols):
            if deg[i, j] < 0:
                continue
            v = int(deg[i, j]) + int(shift[j])
            if best is None or v >= best:
                best, bj = v, j
        rdeg.append(best if best is not None else None)
        piv.append(bj)
    return rdeg, piv


# ---- shifted Popov approximant basis ---------------------------------------

def popov_pmbasis(F: np.ndarray, order: int, shift, p: int, nthreads: int = 1):
    """(appbas, rdeg): the shift-Popov approximant basis (popov_pmbasis,
    mat_lzz_pX_pmbasis.cpp:1527) and its shifted row degree."""
    F = _c64(F)
    m, n, flen = F.shape
    sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
    out = np.zeros((m, m, order + 1), dtype=np.uint64)
    L = int(lib().orc_popov_pmbasis(_p64(out), _pi64(sh), _p64(F), m, n, flen, order, p, nthreads))
    return out[:, :, :max(L, 1)], sh


def is_popov(P: np.ndarray, shift) -> bool:
    """Shift-Popov form (row-wise): pivots on the diagonal (the rightmost entry reaching
    the shifted row degree), monic pivots, and in every column the pivot of strictly
    largest degree."""
    m = P.shape[0]
    rdeg, piv = row_degrees_and_pivots(P, shift)
    if list(piv) != list(range(m)):
        return False
    L = P.shape[2]
    deg = np.full((m, m), -1, dtype=np.int64)
    nz = P != 0
    for d in range(L):
        deg[nz[:, :, d]] = d
    for j in range(m):
        if P[j, j, deg[j, j]] != 1:
            return False
        for i in range(m):
            if i != j and deg[i, j] >= deg[j, j]:
                return False
    return True


# ---- truncated inverse, Dixon lifting --------------------------------------

def inv_trunc(A: np.ndarray, order: int, p: int, nthreads: int = 1):
    """(S, invertible): S = A^-1 mod x^order, shape (n, n, order + 1) (nmod_poly_mat_dixon.c:32)."""
    A = _c64(A)
    n, _, alen = A.shape
    S = np.zeros((n, n, order + 1), dtype=np.uint64)
    ok = int(lib().orc_inv_trunc(_p64(S), _p64(A), n, alen, order, p, nthreads))
    return S, bool(ok)


def dixon(A: np.ndarray, B: np.ndarray, order: int, sigma: int, p: int, nthreads: int = 1):
    """(X, ok): A X = B mod x^sigma by x-adic lifting (nmod_poly_mat_dixon.c:92);
    X has shape (n, m, ceil(sigma / order) * order)."""
    A, B = _c64(A), _c64(B)
    n, _, alen = A.shape
    _, m, blen = B.shape
    L = (sigma + order - 1) // order
    X = np.zeros((n, m, max(L * order, 1)), dtype=np.uint64)
    ok = int(lib().orc_dixon(_p64(X), _p64(A), _p64(B), n, m, alen, blen, order, sigma, p, nthreads))
    return X, bool(ok)


# ---- layout conversions ----------------------------------------------------

def poly_mat_to_mat_poly(P: np.ndarray, order: int, out_cap: int = None):
    """(r, c, len) entry-major -> (out_cap, r, c) coefficient-major, truncated at
    order; returns (array, normalised length)."""
    P = _c64(P)
    r, c, ln = P.shape
    K = min(order, ln)
    out_cap = K if out_cap is None else out_cap
    out = np.zeros((max(out_cap, 0), r, c), dtype=np.uint64)
    L = int(lib().orc_poly_mat_to_mat_poly(_p64(out), out_cap, _p64(P), r, c, ln, ln, order))
    return out, L


def mat_poly_to_poly_mat(M: np.ndarray, order: int, out_cap: int = None):
    """(len, r, c) coefficient-major -> (r, c, out_cap) entry-major, truncated at order."""
    M = _c64(M)
    ln, r, c = M.shape
    K = min(order, ln)
    out_cap = K if out_cap is None else out_cap
    out = np.zeros((r, c, max(out_cap, 0)), dtype=np.uint64)
    lib().orc_mat_poly_to_poly_mat(_p64(out), out_cap, _p64(M), r, c, ln, order)
    return out


# ---- dot products, CRT ------------------------------------------------------

def nmod_vec_dot(v1: np.ndarray, v2: np.ndarray, p: int) -> int:
    v1, v2 = _c64(v1), _c64(v2)
    return int(lib().orc_nmod_vec_dot(_p64(v1), _p64(v2), len(v1), p))


def nmod_vec_dot_multi(u: np.ndarray, v: np.ndarray, p: int, nthreads: int = 1) -> np.ndarray:
    """uv[j] = sum_i u[i] v[i, j] mod p for v of shape (len, k)."""
    u = _c64(u)
    v = _c64(v)
    ln, k = v.shape
    out = np.empty(k, dtype=np.uint64)
    lib().orc_nmod_vec_dot_multi(_p64(out), _p64(u), _p64(v), ln, k, p, nthreads)
    return out


def nmod32_vec_dot(v1: np.ndarray, v2: np.ndarray, p: int) -> int:
    v1 = np.ascontiguousarray(v1, dtype=np.uint32)
    v2 = np.ascontiguousarray(v2, dtype=np.uint32)
    return int(lib().orc_nmod32_vec_dot(_p32(v1), _p32(v2), len(v1), p))


def integer_dot(v1: np.ndarray, v2: np.ndarray) -> int:
    v1, v2 = _c64(v1), _c64(v2)
    res = np.zeros(3, dtype=np.uint64)
    lib().orc_integer_dot(_p64(res), _p64(v1), _p64(v2), len(v1))
    return int(res[0]) | (int(res[1]) << 64) | (int(res[2]) << 128)


def nmod32_vec_mdot(mat: np.ndarray, vec: np.ndarray, p: int) -> np.ndarray:
    mat = np.ascontiguousarray(mat, dtype=np.uint32)
    vec = np.ascontiguousarray(vec, dtype=np.uint32)
    nrows, stride = mat.shape
    out = np.zeros(nrows, dtype=np.uint32)
    lib().orc_nmod32_vec_mdot(_p32(out), _p32(mat), _p32(vec), nrows, len(vec), stride, p)
    return out


def multimod_reduce(x: np.ndarray, primes) -> np.ndarray:
    x = _c64(x)
    pr = _c64(primes)
    out = np.zeros((len(pr), len(x)), dtype=np.uint64)
    lib().orc_multimod_reduce(_p64(out), _p64(x), len(x), _p64(pr), len(pr))
    return out


def multimod_crt(res: np.ndarray, primes, p: int) -> np.ndarray:
    res = _c64(res)
    pr = _c64(primes)
    nb = res.shape[1]
    out = np.zeros(nb, dtype=np.uint64)
    lib().orc_multimod_crt(_p64(out), _p64(res), nb, _p64(pr), len(pr), p)
    return out
