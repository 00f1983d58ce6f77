"""The multi-GPU path's host logic on CPU ranks (gloo, world size 2): scan
shards are disjoint and together form the denser scan, and the job time is
the slowest rank's."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from pisco4cmb_gb300 import synth

    ra, dec, pa = synth.sweep_scan(5000, 2, shard=rank, nshards=world)
    t = bench.max_over_ranks(1.5 + rank, dist, "cpu")  # rank 1 is the slower one
    np.savez(os.path.join(out_dir, "r%d.npz" % rank), ra=ra, dec=dec, pa=pa, t=t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shards_and_timing(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    r = [np.load(tmp_path / ("r%d.npz" % k)) for k in range(world)]
    assert float(r[0]["t"]) == float(r[1]["t"]) == 2.5
    from pisco4cmb_gb300 import synth

    ra1, dec1, _ = synth.sweep_scan(5000, 2)
    # shard 0 of 2 is the plain sweep; shard 1 sits half a sample further in RA
    assert np.array_equal(r[0]["ra"], ra1) and np.array_equal(r[0]["dec"], dec1)
    step = np.deg2rad(360.0 / 4096)
    d = (r[1]["ra"] - r[0]["ra"]) / step
    assert np.allclose(d, 0.5) and np.array_equal(r[1]["dec"], r[0]["dec"])
    assert not np.array_equal(r[0]["pa"], r[1]["pa"])
