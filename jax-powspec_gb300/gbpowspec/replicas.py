"""Multi-GPU replicas: mocks are independent, so ranks shard them with no
data-path collective (no reference counterpart: the reference runs one
process on one device).

One process per GPU (torchrun).  Each rank takes its own share of the mocks
(`shard`), runs them through its own lanes, and the only collectives are
host-side bookkeeping: the slowest rank's time (`max_over_ranks`) for the
whole-job throughput, and gathering the small per-mock P_l arrays on rank 0
for a covariance (`gather_rows`).  Works with the nccl backend (CUDA tensors)
and with gloo (CPU tensors), which is how it is tested without GPUs.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.distributed as dist

__all__ = ["world", "shard", "rank_seed", "max_over_ranks", "gather_rows"]


def world() -> tuple[int, int]:
    """(rank, world size); (0, 1) without an initialised process group."""
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shard(n_items: int, rank: int, size: int) -> np.ndarray:
    """Indices of the items rank `rank` of `size` processes: round-robin, disjoint, covering."""
    if size < 1 or not (0 <= rank < size):
        raise ValueError("bad rank / world size")
    return np.arange(rank, int(n_items), size, dtype=np.int64)


def rank_seed(base: int, rank: int) -> int:
    """A distinct, reproducible seed per rank (catalogues never repeat across ranks)."""
    return int(base) * 1_000_003 + int(rank)


def _device_for_backend():
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(values) -> list:
    """Element-wise maximum of a list of floats over all ranks (identity without a process group)."""
    v = [float(x) for x in values]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return v
    t = torch.tensor(v, dtype=torch.float64, device=_device_for_backend())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def gather_rows(rows: np.ndarray, index: np.ndarray, n_total: int) -> np.ndarray | None:
    """Assemble per-item rows (e.g. P_l of each mock) from every rank on rank 0.

    rows: [len(index), ...] this rank's rows for global items `index`.
    Returns the [n_total, ...] array on rank 0 and None elsewhere.
    """
    rows = np.asarray(rows, dtype=np.float64)
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        out = np.full((n_total,) + rows.shape[1:], np.nan)
        out[np.asarray(index)] = rows
        return out
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, (np.asarray(index), rows))
    if dist.get_rank() != 0:
        return None
    out = np.full((n_total,) + rows.shape[1:], np.nan)
    for idx, r in parts:
        out[idx] = r
    return out
