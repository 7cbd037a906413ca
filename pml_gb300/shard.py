"""Row-sharded polynomial-matrix products over several GPUs, one process per GPU.

The reference computes C = A * B by evaluating every entry of A and B, one
matrix product per evaluation point, and interpolating every entry of C
(flint-extras/src/nmod_poly_mat_extra/mul_geometric.c:78-80 evaluates the
entries, :95-96 is the per-point loop, :104 interpolates).  Row i of C needs
only row i of A and all of B, so the rows of A (and of C) are split over the
ranks: rank g evaluates its own rows of A, evaluates all of B itself (B's
evaluations are recomputed on every rank instead of being exchanged), runs the
per-point products of its rows and interpolates its rows of C.  The only data
exchanged is the result: an all-gather of the row blocks of C, when every rank
wants the whole product.

In the entry-major layout (P[(i*c + j)*len + d]) a block of rows of A or C is
one contiguous range of memory, so a rank's share is the ordinary product
entry point called on a pointer offset: no copy and no strided view.  Remote
data (the gathered blocks of C) always lands in local memory.

The functions take a torch.distributed process group: NCCL for CUDA tensors,
gloo for host tensors (the CPU tests).  `mul` computes one rank's block and is
the GPU product by default.
"""
from __future__ import annotations

from typing import Callable, List, Optional, Tuple


def row_partition(r: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous row ranges [r0, r1) of an r-row matrix for `world` ranks; the first
    r % world ranks get one row more.  Ranks beyond r get empty ranges."""
    if r < 0 or world < 1:
        raise ValueError("need r >= 0 and world >= 1")
    base, extra = divmod(r, world)
    out, r0 = [], 0
    for g in range(world):
        n = base + (1 if g < extra else 0)
        out.append((r0, r0 + n))
        r0 += n
    return out


def _gpu_mul(A_rows, B, p: int, ctx):
    from . import nmod_poly_mat_multiply
    return nmod_poly_mat_multiply(A_rows, B, p, ctx=ctx)


def poly_mat_mul_rows(A, B, p: int, r0: int, r1: int, ctx=None, mul: Optional[Callable] = None):
    """Rows [r0, r1) of C = A * B: A is (r, k, len1) entry-major, B (k, c, len2); returns
    (r1 - r0, c, len1 + len2 - 1).  The row block A[r0:r1] is contiguous, so the product
    runs on it directly."""
    r, k, l1 = A.shape
    k2, c, l2 = B.shape
    if k != k2:
        raise ValueError("inner dimensions differ")
    if not (0 <= r0 <= r1 <= r):
        raise ValueError("row range outside the matrix")
    f = mul if mul is not None else (lambda X, Y, q: _gpu_mul(X, Y, q, ctx))
    return f(A[r0:r1], B, p)


def poly_mat_mul_sharded(A, B, p: int, group=None, ctx=None, gather: bool = True,
                         mul: Optional[Callable] = None):
    """C = A * B with the rows of A split over the ranks of `group` (every rank passes the
    same A and B; it reads only its own rows of A).  Each rank computes its block of rows
    of C; with gather, the blocks are all-gathered so every rank returns the whole C,
    otherwise each rank returns (its block, (r0, r1)).  A rank whose range is empty
    computes nothing and contributes an empty block."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    r, k, l1 = A.shape
    _, c, l2 = B.shape
    clen = l1 + l2 - 1 if (l1 > 0 and l2 > 0) else 0
    parts = row_partition(r, world)
    r0, r1 = parts[rank]
    if r1 > r0:
        block = poly_mat_mul_rows(A, B, p, r0, r1, ctx=ctx, mul=mul)
    else:
        block = torch.zeros((0, c, clen), dtype=torch.int64, device=A.device)
    if not gather:
        return block, (r0, r1)
    # all_gather wants equal shapes: pad every block to the largest row count
    rmax = max(b - a for a, b in parts)
    padded = torch.zeros((rmax, c, clen), dtype=torch.int64, device=block.device)
    if r1 > r0:
        padded[: r1 - r0] = block
    bufs = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(bufs, padded, group=group)
    C = torch.empty((r, c, clen), dtype=torch.int64, device=block.device)
    for g, (a, b) in enumerate(parts):
        if b > a:
            C[a:b] = bufs[g][: b - a]
    return C
