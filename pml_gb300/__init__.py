"""pml_gb300 -- GB300 (sm_103a) implementation of PML's evaluation/interpolation
hot path for polynomial matrices over Z/pZ.

The compute is the CUDA library libpmlg.so (C ABI, include/pmlg.h).  This
module is its host-side mirror of the reference interface: the functions keep
the flint-extras names (nmod_poly_mat_multiply, nmod_poly_mat_mulmid,
nmod_poly_mat_pmbasis, nmod_poly_mat_mbasis, nmod_vec_dot_product, ...) and
their argument meaning, over dense arrays instead of FLINT structs:

* a polynomial matrix is an array of shape (rows, cols, len), entry-major,
  coefficients in [0, p) stored as uint64 (torch.int64 holding the same bits
  on the GPU, numpy.uint64 on the host);
* device tensors are processed on the current torch CUDA stream; numpy arrays
  go through the *_host entry points (copies included).

There is no CPU fallback: every function calls libpmlg.so and raises
PmlgError on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import FORM_AUTO, FORM_CUDA_CORE, FORM_F16_TC, FORM_INT8_TC, PmlgError, PolymatJob, check

__all__ = [
    "Context", "default_context", "PmlgError", "FORM_AUTO", "FORM_CUDA_CORE", "FORM_INT8_TC", "FORM_F16_TC",
    "nmod_mat_mul_batch", "nmod_poly_mat_multiply", "nmod_poly_mat_mulmid", "nmod_poly_mat_multiply_batch",
    "nmod_poly_mat_pmbasis", "nmod_poly_mat_mbasis", "nmod_poly_mat_popov_pmbasis", "nmod_poly_mat_kernel",
    "nmod_poly_mat_kernel_oriented", "nmod_poly_mat_kernel_via_approx",
    "nmod_mat_poly_set_trunc_from_poly_mat", "nmod_poly_mat_set_trunc_from_mat_poly",
    "nmod_poly_mat_inv_trunc", "nmod_poly_mat_dixon", "nmod_vec_dot_product", "nmod32_vec_dot_product",
    "nmod32_vec_mdot", "nmod_vec_dot_product_multi", "nmod_multimod_CRT_reduce", "nmod_multimod_CRT_CRT",
]


class Context:
    """A pmlg_ctx: NTT tables, scratch memory and the pointwise-product form."""

    def __init__(self, device: int = 0, form: int = FORM_AUTO, leaf_order: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.pmlg_ctx_create(C.byref(h), device))
        self.handle = h
        self.device = device
        self.set_form(form)
        if leaf_order:
            self.set_leaf_order(leaf_order)

    def set_form(self, form: int) -> None:
        check(self.lib.pmlg_ctx_set_form(self.handle, form), self.handle)
        self.form = form

    def set_leaf_order(self, order: int) -> None:
        check(self.lib.pmlg_ctx_set_leaf_order(self.handle, order), self.handle)

    def set_tuning(self, on: bool) -> None:
        """PMLG_FORM_AUTO measures the forms per shape class (on) or takes FP16 (off)."""
        check(self.lib.pmlg_ctx_set_tuning(self.handle, 1 if on else 0), self.handle)

    def tuned_form(self, r: int, k: int, c: int, npts: int) -> int:
        """The form AUTO chose for the shape class, 0 (PMLG_FORM_AUTO) if not measured yet."""
        f = self.lib.pmlg_ctx_tuned_form(self.handle, r, k, c, npts)
        if f < 0:
            raise ValueError("shape outside 1..64")
        return f

    def set_batch_graphs(self, on: bool) -> None:
        """Capture repeated batches into CUDA graphs (on, the default) or launch directly."""
        check(self.lib.pmlg_ctx_set_batch_graphs(self.handle, 1 if on else 0), self.handle)

    @property
    def launches(self) -> int:
        return int(self.lib.pmlg_ctx_launch_count(self.handle))

    def check(self, status: int) -> None:
        check(status, self.handle)

    def set_profiling(self, on: bool) -> None:
        """Bracket every kernel launch with CUDA events on its stream (and clear
        earlier records)."""
        check(self.lib.pmlg_ctx_set_profiling(self.handle, 1 if on else 0), self.handle)

    def profile(self) -> dict:
        """{kernel name: (total device ms, launches)} since set_profiling(True)."""
        nmax = 64
        names = C.create_string_buffer(8192)
        ms = (C.c_double * nmax)()
        cnt = (C.c_ulonglong * nmax)()
        n = C.c_int(0)
        check(self.lib.pmlg_ctx_profile_read(self.handle, names, 8192, ms, cnt, nmax, C.byref(n)), self.handle)
        keys = names.value.decode().split("\n")
        return {keys[i]: (ms[i], int(cnt[i])) for i in range(n.value)}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.pmlg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


def _stream_ptr(t) -> int:
    import torch
    return torch.cuda.current_stream(t.device).cuda_stream


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(t) -> int:
    return t.data_ptr() if _is_torch(t) else t.ctypes.data


def _ctx(ctx: Optional[Context], t=None) -> Context:
    if ctx is not None:
        return ctx
    dev = t.device.index if (t is not None and _is_torch(t) and t.device.index is not None) else 0
    return default_context(dev)


def _require_cuda(*ts):
    for t in ts:
        if not (_is_torch(t) and t.is_cuda and t.is_contiguous()):
            raise TypeError("expected contiguous CUDA tensors")


# ---------------------------------------------------------------------------
# L2: batched matrix products mod p
# ---------------------------------------------------------------------------

def nmod_mat_mul_batch(A, B, p: int, ctx: Optional[Context] = None):
    """C[b] = A[b] @ B[b] mod p, uint32 storage (torch.int32 CUDA tensors of shape
    (nb, r, k) and (nb, k, c)); p < 2^30.  Per-point nmod_mat_mul of
    mul_geometric.c:95-96."""
    import torch
    _require_cuda(A, B)
    nb, r, k = A.shape
    nb2, k2, c = B.shape
    assert nb == nb2 and k == k2
    ctx = _ctx(ctx, A)
    out = torch.empty((nb, r, c), dtype=A.dtype, device=A.device)
    ctx.check(ctx.lib.pmlg_nmod_mat_mul_batch_u32(ctx.handle, _ptr(out), _ptr(A), _ptr(B), nb, r, k, c, p,
                                                  _stream_ptr(A)))
    return out


# ---------------------------------------------------------------------------
# L3: products
# ---------------------------------------------------------------------------

def nmod_poly_mat_multiply(A, B, p: int, ctx: Optional[Context] = None, out=None):
    """res = A * B (nmod_poly_mat_multiply, mul.c:19).  A: (r, k, len1), B: (k, c, len2);
    returns (r, c, len1 + len2 - 1).  CUDA tensors run on the current stream;
    numpy arrays use the host-buffer entry point."""
    r, k, l1 = A.shape
    k2, c, l2 = B.shape
    if k != k2:
        raise ValueError("inner dimensions differ")
    clen = l1 + l2 - 1 if (l1 > 0 and l2 > 0) else 0
    ctx = _ctx(ctx, A)
    if _is_torch(A):
        import torch
        _require_cuda(A, B)
        if out is None:
            out = torch.empty((r, c, clen), dtype=torch.int64, device=A.device)
        ctx.check(ctx.lib.pmlg_poly_mat_mul(ctx.handle, _ptr(out), _ptr(A), _ptr(B), r, k, c, l1, l2, p,
                                            _stream_ptr(A)))
        return out
    A = np.ascontiguousarray(A, dtype=np.uint64)
    B = np.ascontiguousarray(B, dtype=np.uint64)
    if out is None:
        out = np.empty((r, c, clen), dtype=np.uint64)
    ctx.check(ctx.lib.pmlg_poly_mat_mul_host(ctx.handle, _ptr(out), _ptr(A), _ptr(B), r, k, c, l1, l2, p, None))
    return out


def nmod_poly_mat_mulmid(A, B, nlo: int, nhi: int, p: int, ctx: Optional[Context] = None,
                         want_length: bool = False):
    """res = (A * B mod x^nhi) div x^nlo (nmod_poly_mat_mulmid, mulmid.c:499).
    Returns the (r, c, nhi - nlo) array, and with want_length the clamped length."""
    r, k, l1 = A.shape
    _, c, l2 = B.shape
    cap = max(nhi - nlo, 0)
    ctx = _ctx(ctx, A)
    n = C.c_int64(0)
    nptr = C.byref(n) if want_length else None
    if _is_torch(A):
        import torch
        _require_cuda(A, B)
        out = torch.empty((r, c, cap), dtype=torch.int64, device=A.device)
        ctx.check(ctx.lib.pmlg_poly_mat_mulmid(ctx.handle, _ptr(out), _ptr(A), _ptr(B), r, k, c, l1, l2, nlo, nhi,
                                               p, nptr, _stream_ptr(A)))
    else:
        A = np.ascontiguousarray(A, dtype=np.uint64)
        B = np.ascontiguousarray(B, dtype=np.uint64)
        out = np.empty((r, c, cap), dtype=np.uint64)
        ctx.check(ctx.lib.pmlg_poly_mat_mulmid_host(ctx.handle, _ptr(out), _ptr(A), _ptr(B), r, k, c, l1, l2, nlo,
                                                    nhi, p, nptr, None))
    return (out, int(n.value)) if want_length else out


def nmod_poly_mat_multiply_batch(jobs, ctx: Optional[Context] = None, out=None):
    """jobs: list of (A, B, p) with CUDA tensors; returns the list of products,
    computed by one pmlg_poly_mat_mul_batch call.  `out`, a list of contiguous int64
    CUDA tensors of the products' shapes, receives them instead of new tensors (a batch
    repeated on the same buffers is replayed from a CUDA graph)."""
    import torch
    if not jobs:
        return []
    ctx = _ctx(ctx, jobs[0][0])
    if out is not None and len(out) != len(jobs):
        raise ValueError("out must hold one tensor per job")
    outs = []
    arr = (PolymatJob * len(jobs))()
    for i, (A, B, p) in enumerate(jobs):
        _require_cuda(A, B)
        r, k, l1 = A.shape
        _, c, l2 = B.shape
        shape = (r, c, l1 + l2 - 1 if l1 and l2 else 0)
        if out is None:
            o = torch.empty(shape, dtype=torch.int64, device=A.device)
        else:
            o = out[i]
            if tuple(o.shape) != shape or o.dtype != torch.int64 or not o.is_cuda or not o.is_contiguous():
                raise ValueError(f"out[{i}] must be a contiguous int64 CUDA tensor of shape {shape}")
        outs.append(o)
        arr[i] = PolymatJob(r, k, c, l1, l2, p, _ptr(A), _ptr(B), _ptr(o))
    ctx.check(ctx.lib.pmlg_poly_mat_mul_batch(ctx.handle, C.cast(arr, C.c_void_p), len(jobs),
                                              _stream_ptr(jobs[0][0])))
    return outs


# ---------------------------------------------------------------------------
# L4: approximant bases
# ---------------------------------------------------------------------------

def _approx(fn_dev, fn_host, F, order: int, shift, p: int, ctx):
    m, n, flen = F.shape
    ctx = _ctx(ctx, F)
    sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
    ln = C.c_int64(0)
    cap = order + 1
    shp = sh.ctypes.data_as(C.POINTER(C.c_int64))
    if _is_torch(F):
        import torch
        _require_cuda(F)
        out = torch.zeros((m, m, cap), dtype=torch.int64, device=F.device)
        ctx.check(fn_dev(ctx.handle, _ptr(out), cap, shp, _ptr(F), m, n, flen, order, p, C.byref(ln),
                         _stream_ptr(F)))
    else:
        F = np.ascontiguousarray(F, dtype=np.uint64)
        out = np.zeros((m, m, cap), dtype=np.uint64)
        ctx.check(fn_host(ctx.handle, _ptr(out), cap, shp, _ptr(F), m, n, flen, order, p, C.byref(ln), None))
    L = max(int(ln.value), 1)
    return out[:, :, :L], sh


def nmod_poly_mat_pmbasis(F, order: int, shift, p: int, ctx: Optional[Context] = None):
    """(appbas, shifted row degree) = nmod_poly_mat_pmbasis(F, order, shift)
    (approximant_basis.c:33).  appbas has shape (m, m, length)."""
    ctx = _ctx(ctx, F)
    return _approx(ctx.lib.pmlg_pmbasis, ctx.lib.pmlg_pmbasis_host, F, order, shift, p, ctx)


def nmod_poly_mat_popov_pmbasis(F, order: int, shift, p: int, ctx: Optional[Context] = None):
    """(appbas, shifted row degree): the shift-Popov approximant basis, canonical
    (popov_pmbasis, mat_lzz_pX_pmbasis.cpp:1527), CUDA tensors only."""
    ctx = _ctx(ctx, F)
    return _approx(ctx.lib.pmlg_popov_pmbasis, None, F, order, shift, p, ctx)


def nmod_poly_mat_mbasis(F, order: int, shift, p: int, ctx: Optional[Context] = None):
    """nmod_poly_mat_mbasis (approximant_basis.c:18), CUDA tensors only."""
    ctx = _ctx(ctx, F)
    return _approx(ctx.lib.pmlg_mbasis, None, F, order, shift, p, ctx)


# ---------------------------------------------------------------------------
# layout conversions
# ---------------------------------------------------------------------------

def nmod_mat_poly_set_trunc_from_poly_mat(P, order: int, ctx: Optional[Context] = None, out=None):
    """Coefficient-major copy (len, r, c) of the entry-major CUDA tensor P (r, c, len),
    truncated at order (nmod_mat_poly_set_from.c:31).  Returns (out, normalised length)."""
    import torch
    _require_cuda(P)
    ctx = _ctx(ctx, P)
    r, c, ln = P.shape
    K = min(order, ln)
    if out is None:
        out = torch.empty((K, r, c), dtype=torch.int64, device=P.device)
    L = C.c_int64(0)
    ctx.check(ctx.lib.pmlg_poly_mat_to_mat_poly(ctx.handle, _ptr(out), out.shape[0], _ptr(P), r, c, ln, ln, order,
                                                C.byref(L), _stream_ptr(P)))
    return out, int(L.value)


def nmod_poly_mat_set_trunc_from_mat_poly(M, order: int, ctx: Optional[Context] = None, out=None):
    """Entry-major copy (r, c, K) of the coefficient-major CUDA tensor M (len, r, c),
    K = min(order, len) (nmod_poly_mat_utils.c:185)."""
    import torch
    _require_cuda(M)
    ctx = _ctx(ctx, M)
    ln, r, c = M.shape
    K = min(order, ln)
    if out is None:
        out = torch.empty((r, c, K), dtype=torch.int64, device=M.device)
    ctx.check(ctx.lib.pmlg_mat_poly_to_poly_mat(ctx.handle, _ptr(out), out.shape[2], _ptr(M), r, c, ln, order,
                                                _stream_ptr(M)))
    return out


ORIENT = {"COL_UPPER": 0, "COL_LOWER": 1, "ROW_UPPER": 2, "ROW_LOWER": 3}


def nmod_poly_mat_kernel_oriented(pmat, p: int, orient: str = "ROW_LOWER", shift=None,
                                  ctx: Optional[Context] = None, cap: Optional[int] = None):
    """nmod_poly_mat_kernel (kernel.c:26) on the (r, c, len) CUDA tensor pmat, form
    ORD_WEAK_POPOV: (ker, pivind, shift_out).  Left kernels (ROW_*) give the
    (nullity, r, length) rows, right kernels (COL_*) the (c, nullity, length)
    columns.  shift None: the default row / column degrees (shift_out is then None)."""
    import torch
    _require_cuda(pmat)
    ctx = _ctx(ctx, pmat)
    r, c, plen = pmat.shape
    o = ORIENT[orient]
    left = o >= 2
    m, n = (r, c) if left else (c, r)
    cap = cap or max(1, (min(m, n) + 1) * max(plen, 1) + 1)
    while True:
        sh = None if shift is None else np.ascontiguousarray(shift, dtype=np.int64).copy()
        piv = np.zeros(max(m, 1), dtype=np.int64)
        ker = torch.zeros((m, m, cap), dtype=torch.int64, device=pmat.device)
        ln, nul = C.c_int64(0), C.c_int64(0)
        st = ctx.lib.pmlg_kernel(ctx.handle, _ptr(ker), cap, C.byref(ln), piv.ctypes.data_as(C.POINTER(C.c_int64)),
                                 sh.ctypes.data_as(C.POINTER(C.c_int64)) if sh is not None else None, _ptr(pmat),
                                 r, c, plen, p, 3, o, C.byref(nul), _stream_ptr(pmat))
        if st == 4 and ln.value > cap:
            cap = int(ln.value)
            continue
        ctx.check(st)
        k, L = int(nul.value), max(int(ln.value), 1)
        out = ker[:k, :, :L] if left else ker[:, :k, :L]
        return out.contiguous(), piv[:k].copy(), (sh[:k].copy() if sh is not None else None)


def nmod_poly_mat_kernel_via_approx(pmat, shift, p: int, ctx: Optional[Context] = None, cap: Optional[int] = None):
    """nmod_poly_mat_kernel_via_approx (kernel.c:146) on a CUDA tensor: (ker, pivind, rdeg)."""
    import torch
    _require_cuda(pmat)
    ctx = _ctx(ctx, pmat)
    m, n, plen = pmat.shape
    cap = cap or max(1, (min(m, n) + 2) * max(plen, 1) + 2)
    while True:
        sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
        piv = np.zeros(max(m, 1), dtype=np.int64)
        ker = torch.zeros((m, m, cap), dtype=torch.int64, device=pmat.device)
        ln, nul = C.c_int64(0), C.c_int64(0)
        st = ctx.lib.pmlg_kernel_via_approx(ctx.handle, _ptr(ker), cap, C.byref(ln),
                                            piv.ctypes.data_as(C.POINTER(C.c_int64)),
                                            sh.ctypes.data_as(C.POINTER(C.c_int64)), _ptr(pmat), m, n, plen, p,
                                            C.byref(nul), _stream_ptr(pmat))
        if st == 4 and ln.value > cap:
            cap = int(ln.value)
            continue
        ctx.check(st)
        k = int(nul.value)
        return ker[:k, :, :max(int(ln.value), 1)].contiguous(), piv[:k].copy(), sh[:k].copy()


# ---------------------------------------------------------------------------
# L5: truncated inverse, Dixon lifting
# ---------------------------------------------------------------------------

def nmod_poly_mat_inv_trunc(A, order: int, p: int, ctx: Optional[Context] = None):
    """(S, invertible): S = A^-1 mod x^order for the (n, n, len) CUDA tensor A
    (nmod_poly_mat_dixon.c:32).  S has shape (n, n, order + 1)."""
    import torch
    _require_cuda(A)
    ctx = _ctx(ctx, A)
    n, _, alen = A.shape
    S = torch.zeros((n, n, order + 1), dtype=torch.int64, device=A.device)
    inv = C.c_int(0)
    ctx.check(ctx.lib.pmlg_inv_trunc(ctx.handle, _ptr(S), _ptr(A), n, alen, order, p, C.byref(inv), _stream_ptr(A)))
    return S, bool(inv.value)


def nmod_poly_mat_dixon(A, B, order: int, sigma: int, p: int, ctx: Optional[Context] = None):
    """(X, ok): A X = B mod x^sigma by x-adic lifting (nmod_poly_mat_dixon.c:92), CUDA
    tensors; X has shape (n, m, ceil(sigma / order) * order)."""
    import torch
    _require_cuda(A, B)
    ctx = _ctx(ctx, A)
    n, _, alen = A.shape
    _, m, blen = B.shape
    xcap = max(1, -(-sigma // order) * order)
    X = torch.zeros((n, m, xcap), dtype=torch.int64, device=A.device)
    ok = C.c_int(0)
    ctx.check(ctx.lib.pmlg_dixon(ctx.handle, _ptr(X), xcap, _ptr(A), _ptr(B), n, m, alen, blen, order, sigma, p,
                                 C.byref(ok), _stream_ptr(A)))
    return X, bool(ok.value)


# ---------------------------------------------------------------------------
# L5: kernel bases
# ---------------------------------------------------------------------------

def nmod_poly_mat_kernel(pmat, shift, p: int, ctx: Optional[Context] = None, cap: Optional[int] = None):
    """Left kernel basis (ROW_LOWER) of the (m, n, len) matrix pmat (a CUDA tensor,
    or a numpy array through the host-buffer entry point):
    nmod_poly_mat_kernel_zls_approx (kernel.c:232).  Returns (ker, pivind, rdeg):
    ker has shape (nullity, m, length), in shift-ordered weak Popov form; pivind
    and rdeg are its shift-pivot indices and shift-row degrees."""
    ctx = _ctx(ctx, pmat)
    dev = _is_torch(pmat)
    if dev:
        import torch
        _require_cuda(pmat)
    else:
        pmat = np.ascontiguousarray(pmat, dtype=np.uint64)
    m, n, plen = pmat.shape
    cap = cap or max(1, (min(m, n) + 1) * max(plen, 1) + 1)
    while True:
        sh = np.ascontiguousarray(shift, dtype=np.int64).copy()
        piv = np.zeros(max(m, 1), dtype=np.int64)
        if dev:
            ker = torch.zeros((m, m, cap), dtype=torch.int64, device=pmat.device)
        else:
            ker = np.zeros((m, m, cap), dtype=np.uint64)
        ln, nul = C.c_int64(0), C.c_int64(0)
        fn = ctx.lib.pmlg_kernel_zls if dev else ctx.lib.pmlg_kernel_zls_host
        st = fn(ctx.handle, _ptr(ker), cap, C.byref(ln), piv.ctypes.data_as(C.POINTER(C.c_int64)),
                sh.ctypes.data_as(C.POINTER(C.c_int64)), _ptr(pmat), m, n, plen, p, C.byref(nul),
                _stream_ptr(pmat) if dev else None)
        if st == 4 and ln.value > cap:   # PMLG_ELEN: the basis is longer than the buffer
            cap = int(ln.value)
            continue
        ctx.check(st)
        k = int(nul.value)
        out = ker[:k, :, :max(int(ln.value), 1)]
        return (out.contiguous() if dev else out.copy()), piv[:k].copy(), sh[:k].copy()


# ---------------------------------------------------------------------------
# L1: dot products, CRT
# ---------------------------------------------------------------------------

def nmod_vec_dot_product(v1, v2, p: int, ctx: Optional[Context] = None) -> int:
    """sum v1[i]*v2[i] mod p, 64-bit entries (nmod_vec_dot_product_unbalanced)."""
    import torch
    _require_cuda(v1, v2)
    ctx = _ctx(ctx, v1)
    res = torch.zeros(1, dtype=torch.int64, device=v1.device)
    ctx.check(ctx.lib.pmlg_nmod_vec_dot(ctx.handle, _ptr(res), _ptr(v1), _ptr(v2), v1.numel(), p, _stream_ptr(v1)))
    return int(res.item()) & (2**64 - 1)


def nmod32_vec_dot_product(v1, v2, p: int, ctx: Optional[Context] = None) -> int:
    """_nmod32_vec_dot_split: 32-bit entries (torch.int32 CUDA tensors)."""
    import torch
    _require_cuda(v1, v2)
    ctx = _ctx(ctx, v1)
    res = torch.zeros(1, dtype=torch.int32, device=v1.device)
    ctx.check(ctx.lib.pmlg_nmod32_vec_dot(ctx.handle, _ptr(res), _ptr(v1), _ptr(v2), v1.numel(), p,
                                          _stream_ptr(v1)))
    return int(res.item()) & 0xffffffff


def nmod32_vec_mdot(mat, vec, p: int, ctx: Optional[Context] = None):
    """_nmod32_vec_mdot_split: mv[i] = sum_j mat[i, j] vec[j] mod p."""
    import torch
    _require_cuda(mat, vec)
    ctx = _ctx(ctx, mat)
    nrows, stride = mat.shape
    out = torch.empty(nrows, dtype=torch.int32, device=mat.device)
    ctx.check(ctx.lib.pmlg_nmod32_vec_mdot(ctx.handle, _ptr(out), _ptr(mat), _ptr(vec), nrows, vec.numel(), stride,
                                           p, _stream_ptr(mat)))
    return out


def nmod_vec_dot_product_multi(u, v, p: int, ctx: Optional[Context] = None):
    """nmod_vec_dot_product_multi: uv[j] = sum_i u[i] v[i, j] mod p."""
    import torch
    _require_cuda(u, v)
    ctx = _ctx(ctx, u)
    ln, k = v.shape
    out = torch.empty(k, dtype=torch.int64, device=u.device)
    ctx.check(ctx.lib.pmlg_nmod_vec_dot_multi(ctx.handle, _ptr(out), _ptr(u), _ptr(v), ln, k, p, _stream_ptr(u)))
    return out


def nmod_multimod_CRT_reduce(x, primes, ctx: Optional[Context] = None):
    """residues[j] = x mod primes[j] (nmod_multimod_CRT_reduce)."""
    import torch
    _require_cuda(x)
    ctx = _ctx(ctx, x)
    pr = np.ascontiguousarray(primes, dtype=np.uint64)
    out = torch.empty((len(pr), x.numel()), dtype=torch.int64, device=x.device)
    ctx.check(ctx.lib.pmlg_multimod_reduce(ctx.handle, _ptr(out), _ptr(x), x.numel(), pr.ctypes.data, len(pr),
                                           _stream_ptr(x)))
    return out


def nmod_multimod_CRT_CRT(residues, primes, p: int, ctx: Optional[Context] = None):
    """out = CRT(residues) mod p (nmod_multimod_CRT_CRT)."""
    import torch
    _require_cuda(residues)
    ctx = _ctx(ctx, residues)
    pr = np.ascontiguousarray(primes, dtype=np.uint64)
    nb = residues.shape[1]
    out = torch.empty(nb, dtype=torch.int64, device=residues.device)
    ctx.check(ctx.lib.pmlg_multimod_crt(ctx.handle, _ptr(out), _ptr(residues), nb, pr.ctypes.data, len(pr), p,
                                        _stream_ptr(residues)))
    return out
