"""The N>1 path of bench.py: replicas only.  Two gloo ranks on CPU check the barrier, the
max-over-ranks timing, the whole-job sum, and that every rank draws its own batch (seed +
rank) with no data exchanged between ranks."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import numpy as np
    import bench
    d = bench.Dist()
    d.barrier()
    t_max = d.max(1.0 + rank)            # slowest rank sets the job time
    total = d.sum(10 * (rank + 1))       # units processed by all ranks
    betas, chis = bench.workload(8, 2026 + rank)
    np.save(os.path.join(out_dir, "r%d.npy" % rank), np.array([t_max, total] + list(betas) + list(chis)))
    d.barrier()
    d.dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    torch = pytest.importorskip("torch")
    import numpy as np
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = np.load(tmp_path / "r0.npy")
    r1 = np.load(tmp_path / "r1.npy")
    assert r0[0] == r1[0] == 2.0            # max over ranks
    assert r0[1] == r1[1] == 30.0           # sum over ranks
    assert not np.allclose(r0[2:10], r1[2:10])   # each replica has its own beta draws
