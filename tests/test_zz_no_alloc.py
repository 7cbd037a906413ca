"""GPU test of pmlg_nmod_vec_dot_multi_noalloc, the entry point that allocates
nothing.  It serves callers that cannot allocate device memory where they
call it: a fixed device-memory budget, or no tolerance for the implicit device
synchronisation of cudaMalloc/cudaFree mid-pipeline.  Its partial sums live in
a file-scope device array instead of context scratch.

The test calls it through the C ABI and compares every column of its output,
bit for bit, with the existing entry point pmlg_nmod_vec_dot_multi and with
the oracle's vector-matrix dot product on the same inputs.  It makes calls in
a row with different data, so a later call cannot profit from what an earlier
one left in the shared array.  The shapes include the two limits of the fixed
array: k = 65536 columns (one chunk of rows, the array exactly full) and a
shape where the array's size, not the row count, bounds the number of row
chunks.  The file name sorts last, so a run that stops at the first failure
has run every other test before this one.  It works alone in a fresh process
too: the first call does the device set-up."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import P998, to_dev

pytestmark = pytest.mark.gpu


def _uv(lib_fn, ctx_handle, u, v, p, stream):
    import torch
    ln, k = v.shape
    out = torch.zeros(k, dtype=torch.int64, device="cuda")
    if ctx_handle is None:
        status = lib_fn(out.data_ptr(), u.data_ptr(), v.data_ptr(), ln, k, p, stream)
    else:
        status = lib_fn(ctx_handle, out.data_ptr(), u.data_ptr(), v.data_ptr(), ln, k, p, stream)
    assert status == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint64)


# (len, k): rows bound the chunks; k = 65536 (a single chunk fills the array); 65536 / k = 32
# chunks is the bound (the row count alone would allow more)
SHAPES = [(3000, 77), (257, 4099), (1000, 65536), (40000, 2048)]


@pytest.mark.parametrize("p", [P998, 2 ** 61 - 1, 18446744073709551557])
def test_noalloc_dot_multi_matches_existing_entry_point(p):
    import torch
    import pml_gb300
    from pml_gb300 import _lib
    L = _lib.load()
    ctx = pml_gb300.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    for call, (ln, k) in enumerate(SHAPES):   # calls in a row, different data each time
        hu = oracle.rand_vec(ln, p, 10 + call)
        hv = oracle.rand_vec(ln * k, p, 20 + call).reshape(ln, k)
        u, v = to_dev(hu), to_dev(hv)
        got = _uv(L.pmlg_nmod_vec_dot_multi_noalloc, None, u, v, p, stream)
        ref = _uv(L.pmlg_nmod_vec_dot_multi, ctx.handle, u, v, p, stream)
        assert np.array_equal(got, ref), f"call {call}"
        assert np.array_equal(got, oracle.nmod_vec_dot_multi(hu, hv, p, nthreads=16)), f"call {call}"
        del u, v
    ctx.close()


def test_noalloc_rejects_more_columns_than_its_scratch():
    """k beyond the fixed maximum (65536 columns) is refused before any device work."""
    import torch
    from pml_gb300 import _lib
    L = _lib.load()
    buf = torch.zeros(16, dtype=torch.int64, device="cuda")
    status = L.pmlg_nmod_vec_dot_multi_noalloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), 1, 65537,
                                               P998, torch.cuda.current_stream().cuda_stream)
    assert status == 9   # PMLG_EUNSUP
    torch.cuda.synchronize()
