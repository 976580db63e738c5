"""Row-block sharding (one rank per GPU): nnz-balanced splits, block
extraction, and the y all-gather, on CPU ranks over gloo.  Each rank's block
is multiplied by the oracle here (the device multiply of a block is the
ordinary single-GPU multiply, covered by the GPU parity tests)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

import morpheus_gb300 as mgb
from morpheus_gb300 import generators as gen
from morpheus_gb300 import partition
from oracle import oracle as O


def _host_block_y(block, x):
    return O.OracleMatrix.from_host(mgb.matrix_to_host(block)).multiply(x)


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 7, 8])
def test_splits_are_balanced(parts):
    A = gen.power_law(20000, seed=41)
    ro = A["row_offsets"].astype(np.int64)
    s = partition.nnz_balanced_splits(ro, parts)
    assert s[0] == 0 and s[-1] == A["nrows"] and len(s) == parts + 1
    assert all(a <= b for a, b in zip(s, s[1:]))
    target = A["nnz"] / parts
    longest = int(np.diff(ro).max())
    for k in range(parts):
        assert abs(int(ro[s[k + 1]] - ro[s[k]]) - target) <= longest + 1


@pytest.mark.parametrize("lens", [[], [0, 0, 0], [5], [3, 0, 0, 9, 1]])
def test_splits_edge_cases(lens):
    ro = np.concatenate([[0], np.cumsum(np.asarray(lens, dtype=np.int64))])
    for parts in (1, 2, 5):
        s = partition.nnz_balanced_splits(ro, parts)
        assert s[0] == 0 and s[-1] == len(lens) and len(s) == parts + 1
        assert all(a <= b for a, b in zip(s, s[1:]))


def test_blocks_reassemble_the_product():
    A = gen.power_law(5000, seed=42)
    x = gen.x_vector(A["ncols"], seed=3)
    M = mgb.matrix_from_host(A, device="cpu")
    full = O.OracleMatrix.from_host(A).multiply(x)
    for world in (1, 2, 3, 5):
        parts = [_host_block_y(partition.local_block(M, r, world)[0], x) for r in range(world)]
        assert np.array_equal(np.concatenate(parts), full)  # same per-row order: bit-exact


def test_bad_block_arguments():
    M = mgb.matrix_from_host(gen.laplacian_2d(8), device="cpu")
    with pytest.raises(mgb.InvalidInputException):
        partition.row_block(M, 10, 5)
    with pytest.raises(mgb.InvalidInputException):
        partition.local_block(M, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        A = gen.power_law(6000, seed=43)
        x = gen.x_vector(A["ncols"], seed=4)
        M = mgb.matrix_from_host(A, device="cpu")
        block, splits = partition.local_block(M, rank, world)
        y_local = torch.from_numpy(_host_block_y(block, x))
        y = partition.allgather_rows(y_local, splits)
        np.save(os.path.join(out_dir, f"y{rank}.npy"), y.numpy())
    finally:
        dist.destroy_process_group()


def test_allgather_two_gloo_ranks(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    A = gen.power_law(6000, seed=43)
    full = O.OracleMatrix.from_host(A).multiply(gen.x_vector(A["ncols"], seed=4))
    for r in range(world):
        assert np.array_equal(np.load(tmp_path / f"y{r}.npy"), full)
