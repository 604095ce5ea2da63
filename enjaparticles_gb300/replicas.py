"""Replicas of the SPH step on the GPUs of one node: one process per GPU.

The step does not shard (one particle system is one graph of dependent
neighbour passes on one GPU), so N GPUs run N independent copies of the
workload.  Ranks meet only around timed regions: a barrier before and after,
and a max over ranks of the measured time.  The process group is NCCL on
GPUs and gloo on the CPU; rendezvous through MASTER_ADDR / MASTER_PORT
(127.0.0.1 unless set), the ranks from RANK / LOCAL_RANK / WORLD_SIZE as
torch.distributed.run sets them.
"""
import os


def env_ranks():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


class Replicas:
    def __init__(self, backend=None, device=None):
        import torch
        self.torch = torch
        self.rank, self.local_rank, self.world = env_ranks()
        self.device = device
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = backend or ("nccl" if device is not None and device.type == "cuda" else "gloo")
            dist.init_process_group(backend, rank=self.rank, world_size=self.world)
            self.dist = dist

    def _sync_device(self):
        if self.device is not None and self.device.type == "cuda":
            self.torch.cuda.synchronize(self.device)

    def barrier(self):
        """Device work of this rank finished, then all ranks here."""
        self._sync_device()
        if self.dist is not None:
            self.dist.barrier()
        self._sync_device()

    def _reduce(self, x, op):
        if self.dist is None:
            return float(x)
        t = self.torch.tensor([float(x)], dtype=self.torch.float64,
                              device=self.device if self.device is not None else "cpu")
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        """Max of x over ranks (timings: the job takes as long as its slowest rank)."""
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.MAX)

    def sum(self, x):
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.SUM)

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
