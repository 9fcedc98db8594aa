"""Several GPUs: the correlator-node path shards by job, one process per GPU.

The reference's manager hands out independent (timeslice x subband) jobs to
correlator nodes one by one (sfxc/src/manager_node.cc:201-257,288-391) and
the output node writes the slices in order (sfxc/src/output_node.cc:68-149).
The same decomposition here: each rank correlates its own jobs on its own
GPU with no data exchange, and rank 0 gathers the output bytes and
concatenates them in job order.  The only collectives are host-side (the
gather of outputs, the maximum of the ranks' timings), over whatever
torch.distributed backend is up (gloo on hosts, NCCL between GPUs).
"""
from . import timebase


def jobs_for_rank(n_jobs, world, rank):
    """Job indices of one rank: dealt round-robin, disjoint and covering."""
    if not 0 <= rank < world:
        raise ValueError("rank outside the world")
    return list(range(rank, n_jobs, world))


def slice_job(job, it):
    """Integration `it` of a multi-integration job as a job of its own (what
    the manager sends a correlator node for one timeslice)."""
    tint = timebase.ticks_from_usec(job["integration_time_us"])
    return dict(job, start_ticks=job["start_ticks"] + it * tint, integration_nr=job.get("integration_nr", 0) + it,
                n_integrations=1, protocols=[[p[it]] for p in job["protocols"]])


def merge_outputs(parts):
    """[(job index, output bytes)] from any ranks -> the bytes in job order."""
    return b"".join(bytes(b) for _, b in sorted(parts, key=lambda p: p[0]))


def gather_outputs(parts, group=None):
    """Collect every rank's [(job index, bytes)] on rank 0 (None elsewhere)."""
    import torch.distributed as dist
    if not dist.is_initialized():
        return list(parts)
    out = [None] * dist.get_world_size(group) if dist.get_rank(group) == 0 else None
    dist.gather_object(list(parts), out, dst=0, group=group)
    if out is None:
        return None
    return [p for rank_parts in out for p in rank_parts]


def max_over_ranks(values, group=None):
    """Element-wise maximum of a list of floats over all ranks."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        return list(values)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor(list(values), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return [float(v) for v in t.cpu()]
