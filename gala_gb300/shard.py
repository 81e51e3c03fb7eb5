"""Host-side logic of the multi-GPU form: orbits are independent, so each rank
(one process per GPU) integrates a contiguous range of them and nothing crosses
between GPUs on the data path.  DOP853 ranges are cut on whole batches of
`nbatch` orbits, because gala integrates a batch as one ODE system (one shared
step size; dop853.pyx:228-245): a batch split across ranks would change the
results.  Timing takes the maximum over ranks; outputs are gathered on the host
in rank order when a caller needs them in one place."""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int, granule: int = 100) -> tuple[int, int]:
    """[start, stop) of the orbits of `rank` among `world` ranks: contiguous,
    disjoint, covering [0, n), cut on multiples of `granule` (only the last range
    may end on a partial granule), the granules spread as evenly as possible."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    if n < 0 or granule < 1:
        raise ValueError("n must be >= 0 and granule >= 1")
    units = (n + granule - 1) // granule
    base, extra = divmod(units, world)
    u0 = rank * base + min(rank, extra)
    u1 = u0 + base + (1 if rank < extra else 0)
    return min(n, u0 * granule), min(n, u1 * granule)


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(x: float) -> float:
    """The maximum of x over all ranks (x itself without a process group)."""
    dist = _dist()
    if dist is None:
        return float(x)
    import torch

    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_orbits(w_local: np.ndarray, axis: int = -1) -> np.ndarray | None:
    """Concatenate every rank's host array along `axis` in rank order; the result
    on rank 0, None elsewhere (the array itself without a process group)."""
    dist = _dist()
    if dist is None:
        return w_local
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, np.asarray(w_local))
    return np.concatenate(parts, axis=axis) if dist.get_rank() == 0 else None
