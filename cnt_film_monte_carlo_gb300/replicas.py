"""Replicas on several GPUs, one process per GPU: the only exchange of the path.

Excitons are independent given the read-only neighbour rows, so N GPUs run N replicas of the
film(s) with different Philox keys (replica r of a film whose seed is s uses the 64-bit key
r * 2^32 + s, so every (film, replica) pair has its own key) and nothing crosses GPUs while they
run.  The exchange comes once, at the end: the MSD sums of every (step, batch) and the exciton
counts are combined over replicas (the final reduction of kubo_save_avg_dispalcement_squared,
src/monte_carlo/monte_carlo.cpp:382-409, over the union of the replicas' excitons; batches are
concatenated so the diffusion fit sees every replica's batches), hop counters are summed, and a
timing is the slowest replica's.  Works with any torch.distributed backend (gloo on CPU, nccl).
"""
from __future__ import annotations

import numpy as np


def replica_seed(seed: int, rank: int) -> int:
    """Philox key of replica ``rank`` of a film seeded ``seed``: the rank in the upper 32 bits of
    the 64-bit key, the film's seed (below 2^32) in the lower 32.  Films with distinct seeds on
    any replicas never share a key, so their streams never overlap; replica 0 keeps the film's
    own seed, so a one-GPU run is unchanged."""
    seed, rank = int(seed), int(rank)
    if not 0 <= seed < (1 << 32):
        raise ValueError(f"replica_seed: film seed {seed} outside [0, 2^32)")
    if not 0 <= rank < (1 << 32):
        raise ValueError(f"replica_seed: rank {rank} outside [0, 2^32)")
    return (rank << 32) | seed


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def _device():
    import torch

    dist = _dist()
    if dist is not None and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def gather_batches(msd_batches: np.ndarray, counts: np.ndarray):
    """Concatenate every replica's batches: msd [n_steps][B][3] and counts [B] of this replica ->
    msd [n_steps][B * world][3] and counts [B * world], replica-major (the same on every rank)."""
    import torch

    dist = _dist()
    m = np.ascontiguousarray(msd_batches, dtype=np.float64)
    c = np.ascontiguousarray(counts, dtype=np.int64)
    if dist is None or dist.get_world_size() == 1:
        return m, c
    dev = _device()
    w = dist.get_world_size()
    tm = torch.from_numpy(m).to(dev)
    tc = torch.from_numpy(c).to(dev)
    gm = [torch.empty_like(tm) for _ in range(w)]
    gc = [torch.empty_like(tc) for _ in range(w)]
    dist.all_gather(gm, tm)
    dist.all_gather(gc, tc)
    return (np.concatenate([x.cpu().numpy() for x in gm], axis=1),
            np.concatenate([x.cpu().numpy() for x in gc]))


def sum_msd(msd: np.ndarray) -> np.ndarray:
    """MSD sums (any shape) added over replicas."""
    import torch

    dist = _dist()
    m = np.ascontiguousarray(msd, dtype=np.float64)
    if dist is None or dist.get_world_size() == 1:
        return m
    t = torch.from_numpy(m.copy()).to(_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def job_timing(device_s: float, wall_s: float, hops: float):
    """(slowest replica's device seconds, slowest wall seconds, hops of all replicas)."""
    import torch

    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(device_s), float(wall_s), float(hops)
    dev = _device()
    mx = torch.tensor([device_s, wall_s], dtype=torch.float64, device=dev)
    sm = torch.tensor([float(hops)], dtype=torch.float64, device=dev)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return mx[0].item(), mx[1].item(), sm[0].item()
