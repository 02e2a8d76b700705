"""Replicas: one process per GPU running its own copy of the workload.

The reference has no distributed backend, and the hot path does not shard
below a case (a domain decomposition would need a halo exchange per stage and
a minimum-dt reduction; it is not built).  Independent cases and parameter
sweeps are replicas: no collective touches the data path; the only
collectives are a barrier around the timed region and the reductions of the
ranks' times and counts.  Ranks, world size and the rendezvous come from the
torchrun environment (RANK, LOCAL_RANK, WORLD_SIZE, MASTER_ADDR/PORT).
"""

import os


def env():
    """(rank, local rank, world size) from the launcher's environment."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class Replicas:
    """backend: "nccl" (one GPU per rank) or "gloo" (CPU, tests); a single
    process needs none.  cuda: synchronise the rank's GPU at barriers."""

    def __init__(self, backend="nccl", cuda=True):
        import torch
        self.rank, self.local, self.world = env()
        self.cuda = cuda
        self.torch = torch
        self.dist = None
        if cuda:
            torch.cuda.set_device(self.local)
        if self.world > 1:
            import torch.distributed as dist
            kw = {"device_id": torch.device("cuda", self.local)} if backend == "nccl" else {}
            dist.init_process_group(backend, **kw)
            self.dist = dist
        self.device = torch.device("cuda", self.local) if cuda else torch.device("cpu")

    def barrier(self):
        if self.dist:
            self.dist.barrier()
        if self.cuda:
            self.torch.cuda.synchronize()

    def _reduce(self, x, op):
        if not self.dist:
            return float(x)
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, self.dist.ReduceOp.MAX if self.dist else None)

    def sum(self, x):
        return self._reduce(x, self.dist.ReduceOp.SUM if self.dist else None)

    def rate(self, units, seconds):
        """Whole-job throughput: the units all ranks processed over the
        slowest rank's time."""
        return self.sum(units) / self.max(seconds)

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None
