"""CPU, world_size 2 (gloo): the replica form of the path.

Paths are independent and the bench shards a frame's samples across ranks
with no data-path collective.  Two gloo ranks each render their own sample
chunks with the oracle; the sum of their films equals one process rendering
every chunk, and the max-over-ranks timing reduction works.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, str(REPO))
    import bench
    from oracle import pyoracle as O
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, cam = S.cornell_icosphere(1)
    osc = O.OracleScene(sc)
    k, n_chunks = 2, 4  # 8 spp in chunks of 2
    film = np.zeros((8, 8, 3), np.float64)
    for step in range(2):
        c = bench.sample_chunk(step, rank, world, n_chunks)
        job = N.job_desc(0, cam, 8, 8, 4, 2, 4, seed=3, spp_begin=c * k, spp_end=c * k + k)
        m, _ = osc.render(job, threads=1)
        film += m.astype(np.float64) * k
    t = bench.max_over_ranks(float(rank + 1), True)
    np.save(os.path.join(out_dir, f"film{rank}.npy"), film)
    np.save(os.path.join(out_dir, f"t{rank}.npy"), np.array([t]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_cover_the_frame(tmp_path):
    world = 2
    port = 29500 + (os.getpid() % 1000)
    mp.spawn(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    films = [np.load(tmp_path / f"film{r}.npy") for r in range(world)]
    times = [float(np.load(tmp_path / f"t{r}.npy")[0]) for r in range(world)]
    assert times == [2.0, 2.0]
    sys.path.insert(0, str(REPO))
    from oracle import pyoracle as O
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    sc, cam = S.cornell_icosphere(1)
    job = N.job_desc(0, cam, 8, 8, 4, 2, 4, seed=3)
    full, _ = O.OracleScene(sc).render(job, threads=1)
    total = (films[0] + films[1]) / 8.0
    np.testing.assert_allclose(total, full, rtol=1e-5, atol=1e-6)
