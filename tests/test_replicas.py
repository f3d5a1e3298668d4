"""bench.py on N > 1 ranks (torchrun, one replica of the solve per rank): the job's time is the
slowest rank's, value = solves of all ranks / that time, and the reference arm runs on rank 0
only.  Two gloo ranks on the CPU."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r's own times (ms): the mixed solve, the FP64 solve, the end-to-end solve
        out[rank] = bench.max_over_ranks([10.0 + rank, 20.0 - rank, 30.0 + 2 * rank], "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
        got = dict(out)
    assert got[0] == got[1] == [11.0, 20.0, 32.0]
    # the whole job: two replicas' solves over the slowest rank's time
    assert bench.aggregate_rate(2, 11.0) == 2 * 1e3 / 11.0


def test_reference_arm_other_ranks_do_nothing(capsys):
    class Args:
        steps, warmup = 1, 0
    bench.run_reference(Args(), 1, 2)
    assert capsys.readouterr().out == ""
