"""Multi-process runs: one process per GPU, each an independent replica.

The path shards into independent queries and independent trees, so ranks
share nothing on the data path ("replicas only", weak scaling): each rank
builds and queries its own seeded copy of the workload.  The only collectives
are a barrier around the timed region and the maximum over ranks of the
measured time; the whole-job rate is every rank's units over that maximum.
Read RANK / WORLD_SIZE / LOCAL_RANK / MASTER_* from the environment as
torchrun sets them."""

import os


def env():
    """(rank, world_size, local_rank) of this process (single process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base, rank):
    """Seed of a rank's copy of a seeded input array (rank 0 keeps the base)."""
    return base + 1000 * rank


def whole_job_rate(units_per_rank, seconds_max, world):
    """Units per second of the whole job: all ranks' units over the slowest rank's time."""
    return units_per_rank * world / seconds_max


class Replicas:
    """Process group of the replicas.  backend: "nccl" for GPU ranks, "gloo"
    for host-only ranks (tests); device: the CUDA device of this rank, or
    None for host tensors."""

    def __init__(self, backend="nccl", device=None):
        self.rank, self.world, self.local = env()
        self.device = device
        self._dist = None
        if self.world > 1:
            import torch.distributed as dist

            if not dist.is_initialized():
                dist.init_process_group(backend)
            self._dist = dist

    def _sync(self):
        if self.device is not None:
            import torch

            torch.cuda.synchronize(self.device)

    def barrier(self):
        """Device work of this rank finished, then all ranks meet."""
        self._sync()
        if self._dist is not None:
            self._dist.barrier()
        self._sync()

    def _reduce(self, x, op):
        if self._dist is None:
            return float(x)
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64,
                         device=self.device if self.device is not None else "cpu")
        self._dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, None if self._dist is None else self._dist.ReduceOp.MAX)

    def sum(self, x):
        return self._reduce(x, None if self._dist is None else self._dist.ReduceOp.SUM)

    def close(self):
        if self._dist is not None and self._dist.is_initialized():
            self._dist.destroy_process_group()
