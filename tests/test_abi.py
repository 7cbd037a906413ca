"""CPU tests of the drop-in boundary: libpmlg.so builds for sm_103a, loads,
and exports every entry point that include/pmlg.h declares.  No compute call
is made (there may be no GPU)."""
from __future__ import annotations

import ctypes
import re
import subprocess

from conftest import ROOT


def header_symbols():
    text = (ROOT / "include" / "pmlg.h").read_text()
    return re.findall(r"PMLG_API\s+[\w\s\*]+?\b(pmlg_\w+)\s*\(", text)


def test_header_declares_the_path():
    names = set(header_symbols())
    for required in ["pmlg_ctx_create", "pmlg_nmod_mat_mul_batch_u32", "pmlg_poly_mat_mul", "pmlg_poly_mat_mulmid",
                     "pmlg_pmbasis", "pmlg_mbasis", "pmlg_nmod_vec_dot", "pmlg_nmod32_vec_dot",
                     "pmlg_multimod_reduce", "pmlg_multimod_crt", "pmlg_poly_mat_mul_batch"]:
        assert required in names


def test_library_exports_every_symbol():
    from pml_gb300 import _lib
    L = _lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(pmlg_\w+)", out))
    for name in header_symbols():
        assert name in exported, name
        assert isinstance(getattr(L, name), ctypes._CFuncPtr)
    # the Python binding knows every declared entry point
    assert set(header_symbols()) <= set(_lib.SIGNATURES)


def test_library_is_sm103a():
    from pml_gb300 import _lib, _build
    _lib.load()
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.NVCC_FLAGS)
    assert _lib.LIB_PATH.stat().st_size > 0


def test_status_strings_without_gpu():
    from pml_gb300 import _lib
    L = _lib.load()
    assert L.pmlg_strerror(0) == b"ok"
    assert L.pmlg_strerror(5) == b"output overlaps an input"
    # argument checks happen before any device work
    assert L.pmlg_ctx_create(None, 0) == 1


def test_no_cpu_fallback_in_package():
    """The product package never imports the oracle."""
    for f in (ROOT / "pml_gb300").rglob("*.py"):
        src = f.read_text()
        assert "import oracle" not in src and "from oracle" not in src, f


def test_follow_on_entry_points_reject_bad_arguments_without_gpu():
    """The kernel-basis, Popov, truncated-inverse, Dixon and layout entry points
    check their arguments before touching a device: a null context is EINVAL."""
    import ctypes as C
    from pml_gb300 import _lib
    L = _lib.load()
    i64 = C.c_int64(0)
    ic = C.c_int(0)
    assert L.pmlg_kernel_zls(None, None, 1, C.byref(i64), None, None, None, 1, 1, 1, 7, C.byref(i64), None) == 1
    assert L.pmlg_kernel_zls_host(None, None, 1, C.byref(i64), None, None, None, 1, 1, 1, 7, C.byref(i64),
                                  None) == 1
    assert L.pmlg_popov_pmbasis(None, None, 2, None, None, 1, 1, 1, 1, 7, None, None) == 1
    assert L.pmlg_inv_trunc(None, None, None, 1, 1, 4, 7, C.byref(ic), None) == 1
    assert L.pmlg_dixon(None, None, 8, None, None, 1, 1, 1, 1, 4, 8, 7, C.byref(ic), None) == 1
    assert L.pmlg_poly_mat_to_mat_poly(None, None, 4, None, 1, 1, 4, 4, 4, None, None) == 1
    assert L.pmlg_mat_poly_to_poly_mat(None, None, 4, None, 1, 1, 4, 4, None) == 1
