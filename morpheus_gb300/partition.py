"""Row-block partition of a CSR matrix across ranks (one process per GPU).

Rows of y = A*x are independent, so a matrix is cut into contiguous row
blocks holding (nearly) equal numbers of nonzeros -- the split the reference
makes for its OpenMP COO multiply
(core/src/impl/Coo/OpenMP/Morpheus_Multiply_Impl.hpp:69-106) -- x is
replicated, and every rank computes its block of y with no communication.
An iterative method that needs the whole y as its next x all-gathers the
blocks (allgather_rows), the only exchange of the path.

The split and the block extraction are host logic; the per-rank multiply is
the ordinary device multiply on the block.
"""
from __future__ import annotations

import numpy as np
import torch

from .containers import CsrMatrix
from .exceptions import InvalidInputException


def nnz_balanced_splits(row_offsets, parts: int) -> list[int]:
    """Row boundaries b[0] = 0 <= b[1] <= ... <= b[parts] = nrows such that
    block k (rows b[k]..b[k+1]) starts at the first row whose first entry is
    at or after k * nnz / parts.  Every block then holds nnz/parts entries
    give or take one row; rows are never split."""
    if parts < 1:
        raise InvalidInputException("parts must be >= 1")
    ro = row_offsets.cpu().numpy() if isinstance(row_offsets, torch.Tensor) else np.asarray(row_offsets)
    ro = ro.astype(np.int64)
    n = ro.size - 1
    if n < 0:
        raise InvalidInputException("row_offsets must hold nrows + 1 entries")
    nnz = int(ro[-1]) if n >= 0 else 0
    targets = (np.arange(1, parts, dtype=np.int64) * nnz) // parts
    inner = np.searchsorted(ro[:n], targets, side="left") if n > 0 else np.zeros(parts - 1, np.int64)
    return [0] + [int(b) for b in np.minimum(inner, n)] + [n]


def row_block(A: CsrMatrix, r0: int, r1: int) -> CsrMatrix:
    """Rows r0..r1 of A as a CSR matrix of r1 - r0 rows and A.ncols() columns
    (columns keep their global numbering, so the block multiplies the
    replicated x)."""
    if not 0 <= r0 <= r1 <= A.nrows():
        raise InvalidInputException(f"row block [{r0}, {r1}) outside 0..{A.nrows()}")
    ro = A.row_offsets()
    e0, e1 = int(ro[r0].item()), int(ro[r1].item())
    local_ro = (ro[r0:r1 + 1] - e0).to(torch.int32)
    return CsrMatrix(r1 - r0, A.ncols(), e1 - e0, local_ro, A.column_indices()[e0:e1].clone(),
                     A.values()[e0:e1].clone(), dtype=A.dtype, device=A.device)


def local_block(A: CsrMatrix, rank: int, world: int) -> tuple[CsrMatrix, list[int]]:
    """(this rank's row block, the boundaries of all blocks)."""
    if not 0 <= rank < world:
        raise InvalidInputException(f"rank {rank} outside a world of {world}")
    splits = nnz_balanced_splits(A.row_offsets(), world)
    return row_block(A, splits[rank], splits[rank + 1]), splits


def allgather_rows(y_local: torch.Tensor, splits: list[int], group=None) -> torch.Tensor:
    """Concatenate every rank's block of y (block k has splits[k+1] - splits[k]
    entries) into the full vector on every rank, with one all_gather of
    equal-sized padded blocks."""
    import torch.distributed as dist
    world = len(splits) - 1
    sizes = [splits[k + 1] - splits[k] for k in range(world)]
    rank = dist.get_rank(group)
    if y_local.numel() != sizes[rank]:
        raise InvalidInputException(f"rank {rank} holds {y_local.numel()} rows, its block has {sizes[rank]}")
    width = max(sizes) if sizes else 0
    padded = torch.zeros(width, dtype=y_local.dtype, device=y_local.device)
    padded[:y_local.numel()] = y_local
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    return torch.cat([parts[k][:sizes[k]] for k in range(world)])
