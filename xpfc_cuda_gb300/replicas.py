"""Replica runs over several GPUs of one node (one process per GPU).

The reference splits one grid over the GPUs of a node (cuFFT-Xt slabs,
main.cu:109-113).  With one GPU per solve here, N GPUs run N independent
solves: each rank advances its own field (its own seeds), no data crosses
ranks, and a job's throughput is the grid points all ranks advanced divided by
the slowest rank's time.
"""
import os


def env():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Group:
    """Barrier and max-reduction over the ranks (a no-op for one process)."""

    def __init__(self, backend="nccl", device=None):
        self.world, self.rank, self.local = env()
        self.dist = None
        self.device = device
        if self.world > 1:
            import torch.distributed as dist
            if backend == "nccl":
                import torch
                dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            else:
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device or "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.dist:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device or "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def throughput(units_per_rank, seconds, group):
    """Whole-job units per second: all ranks' units over the slowest time."""
    return group.sum(units_per_rank) / group.max(seconds)
