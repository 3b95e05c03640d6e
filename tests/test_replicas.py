"""The sharded (one process per GPU) host path on CPU with gloo, world size 2:
slice ranges, result collection on rank 0 and the max-over-ranks timing."""
import os
import socket

import numpy as np
import pytest

from lprec_gb300.replicas import gather_slices, max_over_ranks, slice_range


def test_slice_ranges_cover_once():
    for S in (1, 2, 5, 128, 129):
        for world in (1, 2, 3, 8):
            got = [slice_range(S, world, r) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == S
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        slice_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, S, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import lprec_oracle as O
    tr = O.Transform(32, 48, S, 'ramp', 16, 'cubic')
    rng = np.random.default_rng(4)
    f = rng.random((S, 32, 32))
    a, b = slice_range(S, world, rank)
    local = tr.fwd(f[a:b])                        # this rank's slices only
    full = gather_slices(local, S)
    t = max_over_ranks(1.0 + rank)                # every rank sees the slowest rank's time
    if rank == 0:
        np.savez(out_path, full=full, t=t)
    else:
        assert full is None and t == world
    dist.destroy_process_group()


def test_two_rank_gloo_shard_and_gather(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    S, world = 5, 2
    out = str(tmp_path / "r0.npz")
    mp.start_processes(_worker, args=(world, _free_port(), S, out), nprocs=world, start_method="spawn")
    z = np.load(out)
    from oracle import lprec_oracle as O
    tr = O.Transform(32, 48, S, 'ramp', 16, 'cubic')
    f = np.random.default_rng(4).random((S, 32, 32))
    assert np.array_equal(z['full'], tr.fwd(f))
    assert float(z['t']) == 2.0


def test_single_process_fallbacks():
    x = np.arange(6.0).reshape(2, 3)
    assert gather_slices(x, 2) is not None
    assert max_over_ranks(3.5) == 3.5
