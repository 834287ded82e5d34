"""The multi-GPU path on CPU: two replica processes over gloo (world size 2).

Replicas never exchange anything while they run; these tests check the host-side exchange at the
end: MSD sums added over replicas, batches gathered for the diffusion fit (equal to one process
fitting the concatenated batches), and the job timing (slowest replica, all replicas' hops).
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_data(rank, n_steps=40, batches=8):
    rng = np.random.default_rng(100 + rank)
    t = np.arange(1, n_steps + 1) * 1e-12
    slope = np.array([2.0e-4, 1.5e-4, 1e-6]) * (1.0 + 0.1 * rank)
    counts = np.full(batches, 64 + rank, dtype=np.int64)
    msd = (2 * slope[None, None, :] * t[:, None, None] * counts[None, :, None]
           * (1 + 0.05 * rng.standard_normal((n_steps, batches, 3))))
    return msd, counts, t


FILMS = 256


def _worker(rank, world, port, out_dir):
    import sys

    import torch

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from cnt_film_monte_carlo_gb300 import diffusion, replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    msd, counts, t = _replica_data(rank)
    total = replicas.sum_msd(msd.sum(axis=1))
    gm, gc = replicas.gather_batches(msd, counts)
    D, ci = diffusion.fit_counts(gm, gc, t)
    dev, wall, hops = replicas.job_timing(1.0 + rank, 2.0 - rank, 1000 * (rank + 1))
    # the Philox keys of this replica's films (bench.py seeds film i with 1 + i), gathered: no two
    # (film, replica) pairs may share a key
    keys = torch.tensor([replicas.replica_seed(1 + i, rank) for i in range(FILMS)], dtype=torch.int64)
    all_keys = [torch.empty_like(keys) for _ in range(world)]
    dist.all_gather(all_keys, keys)
    np.savez(os.path.join(out_dir, f"r{rank}.npz"), total=total, gm=gm, gc=gc, D=D, ci=ci,
             timing=np.array([dev, wall, hops]), keys=torch.cat(all_keys).numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_over_gloo(tmp_path):
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    from cnt_film_monte_carlo_gb300 import diffusion

    res = [dict(np.load(tmp_path / f"r{r}.npz")) for r in range(world)]
    data = [_replica_data(r) for r in range(world)]
    want_total = sum(m.sum(axis=1) for m, _, _ in data)
    want_m = np.concatenate([m for m, _, _ in data], axis=1)
    want_c = np.concatenate([c for _, c, _ in data])
    D, ci = diffusion.fit_counts(want_m, want_c, data[0][2])
    for r in res:  # every rank holds the same combined result
        np.testing.assert_allclose(r["total"], want_total, rtol=1e-15)
        np.testing.assert_array_equal(r["gm"], want_m)
        np.testing.assert_array_equal(r["gc"], want_c)
        np.testing.assert_allclose(r["D"], D, rtol=1e-14)
        np.testing.assert_allclose(r["ci"], ci, rtol=1e-14)
        np.testing.assert_array_equal(r["timing"], [2.0, 2.0, 3000.0])
        assert len(r["keys"]) == world * FILMS and len(np.unique(r["keys"])) == world * FILMS
        np.testing.assert_array_equal(r["keys"][:FILMS], 1 + np.arange(FILMS))  # replica 0: the films' seeds


def test_single_process_is_identity():
    from cnt_film_monte_carlo_gb300 import replicas

    msd, counts, _ = _replica_data(0)
    m, c = replicas.gather_batches(msd, counts)
    assert np.array_equal(m, msd) and np.array_equal(c, counts)
    assert np.array_equal(replicas.sum_msd(msd), msd)
    assert replicas.job_timing(1.5, 2.5, 10) == (1.5, 2.5, 10.0)


def test_replica_keys_distinct_and_bounded():
    from cnt_film_monte_carlo_gb300 import replicas

    keys = {replicas.replica_seed(s, r) for s in range(300) for r in range(8)}
    assert len(keys) == 300 * 8
    assert replicas.replica_seed(5, 0) == 5 and replicas.replica_seed(5, 1) == (1 << 32) + 5
    assert all(k < (1 << 64) for k in keys)
    for bad in ((-1, 0), (1 << 32, 0), (0, -1), (0, 1 << 32)):
        with pytest.raises(ValueError):
            replicas.replica_seed(*bad)
