"""Replicas on several processes: the end-of-run gather of bins (the reference's
MPI gather, include/utils/mpi.hpp:29-104) over torch.distributed, two gloo ranks on CPU."""
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, size, port, out):
    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from dqmc_gb300 import parallel

    assert parallel.init("gloo") == (rank, size)
    local = np.full((2 + rank, 3), float(rank))  # uneven bin counts per rank
    got = parallel.gather_bins(local)
    if rank == 0:
        np.save(out, got)
    else:
        assert got is None
    import torch.distributed as dist

    dist.destroy_process_group()


def test_gather_bins_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as tmp

    out = str(tmp_path / "bins.npy")
    tmp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    assert got.shape == (5, 3)
    np.testing.assert_array_equal(got[:, 0], [0, 0, 1, 1, 1])


def test_single_process_gets_its_own_bins():
    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    from dqmc_gb300 import parallel

    b = np.arange(6.0).reshape(2, 3)
    np.testing.assert_array_equal(parallel.gather_bins(b), b)
