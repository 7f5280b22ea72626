"""Whole-job figures of a multi-GPU run.

The path tracer does not shard a frame across GPUs: under torchrun every rank renders its
own replica of the workload (weak scaling, no data-path collective).  Rank 0 reports the
units all ranks processed over the slowest rank's time, which takes two reductions at the
end of the timed region.  Works on any initialised process group (NCCL on the GPUs, gloo
on CPU in the tests)."""
import torch


def aggregate(total_ms: float, rays: int, paths: int, device) -> tuple:
    """(max over ranks of total_ms, sum of rays, sum of paths); the inputs unchanged when
    no process group is initialised or it has one rank."""
    import torch.distributed as td
    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return float(total_ms), int(rays), int(paths)
    t = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    r = torch.tensor([float(rays), float(paths)], device=device, dtype=torch.float64)
    td.all_reduce(r)
    return float(t.item()), int(r[0].item()), int(r[1].item())
