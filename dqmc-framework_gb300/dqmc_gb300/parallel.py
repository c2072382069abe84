"""Replicas on several GPUs: the reference's end-of-run gather of bins.

The reference runs one Markov chain per MPI rank and, after the measurement,
gathers every rank's bins on the master (include/utils/mpi.hpp:29-104) before
the analysis.  The sweep itself never exchanges data, so here each process
(one per GPU, launched by torchrun) runs its own batch of walkers and the bins
are gathered once at the end through torch.distributed (NCCL or gloo): no
collective touches the data path.
"""
from __future__ import annotations

import os

import numpy as np


def world() -> tuple[int, int]:
    """(rank, world size) of a torchrun launch, (0, 1) otherwise."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def init(backend: str | None = None) -> tuple[int, int]:
    """Join the process group of a torchrun launch (no-op for one process)."""
    rank, size = world()
    if size > 1:
        import torch.distributed as dist

        if not dist.is_initialized():
            if backend is None:
                import torch

                backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend)
    return rank, size


def gather_bins(local) -> np.ndarray | None:
    """Every rank's bins concatenated in rank order on rank 0 (None on the others);
    a single process gets its own bins back."""
    local = np.asarray(local)
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is always present with this package
        return local
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return local
    rank = dist.get_rank()
    parts = [None] * dist.get_world_size() if rank == 0 else None
    dist.gather_object(local, parts, dst=0)
    return np.concatenate(parts) if rank == 0 else None
