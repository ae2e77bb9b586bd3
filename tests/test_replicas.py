"""Replica bookkeeping across ranks (gloo, world size 2, CPU)."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from mri_recon_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank 1 is the slow one: 2 s for 10 iterations against 1 s on rank 0
    tput, smax = replicas.job_throughput(10, 1.0 + rank)
    out[rank] = (tput, smax, replicas.world())
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_uses_slowest_rank():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    for r in (0, 1):
        tput, smax, w = res[r]
        assert w == 2
        assert smax == 2.0
        assert abs(tput - 10.0) < 1e-12   # 2 ranks x 10 iterations / 2 s


def test_single_process_is_identity():
    from mri_recon_gb300 import replicas
    assert replicas.world() == 1
    assert replicas.job_throughput(7, 0.5) == (14.0, 0.5)
