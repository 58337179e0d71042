"""The multi-rank path on CPU: two gloo ranks each evaluate their contiguous cell range (with the oracle,
standing in for one GPU each) and the gathered result equals the single-process one; timings reduce with
max over ranks, as bench.py does."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from combustion_gb300.sharding import cell_range


def test_cell_ranges_partition():
    for n in (0, 1, 7, 1000, 1 << 22):
        for world in (1, 2, 3, 8):
            ranges = [cell_range(n, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [h - l for l, h in ranges]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import util
    from combustion_gb300 import synthetic
    from combustion_gb300.sharding import cell_range, reduce_max
    n = 1000
    lo, hi = cell_range(n, world, rank)
    o = util.loaded_oracle("k10")
    cells = synthetic.generate_cells(10, hi - lo, "k10", offset=lo)
    out = torch.from_numpy(o.rates(o.rates_inputs(cells)))
    parts = [torch.zeros((out.shape[0], cell_range(n, world, r)[1] - cell_range(n, world, r)[0]), dtype=torch.float64)
             for r in range(world)]
    dist.all_gather(parts, out)
    t = reduce_max(float(rank + 1))
    if rank == 0:
        np.save(os.path.join(out_dir, "gathered.npy"), torch.cat(parts, dim=1).numpy())
        np.save(os.path.join(out_dir, "tmax.npy"), np.array([t]))
    dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process(tmp_path):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    gathered = np.load(tmp_path / "gathered.npy")
    import util
    from combustion_gb300 import synthetic
    o = util.loaded_oracle("k10")
    whole = o.rates(o.rates_inputs(synthetic.generate_cells(10, 1000, "k10")))
    assert np.array_equal(gathered, whole)
    assert np.load(tmp_path / "tmax.npy")[0] == world
