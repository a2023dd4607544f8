"""Instance sharding across GPUs: one process per GPU (torchrun), no data-path collective.

A network never spans GPUs (splitting one by neuron range would need a spike exchange every
step).  What spreads over GPUs are independent units: the replicas of the headline network, the
networks of a batch, the jobs of a served stream.  Units are assigned to ranks by a deterministic
bin packing of their weights (device footprint, or work), computed identically on every rank, so
no rank sends another anything before or during the run.  The only exchange is host-side
reporting at the end: the total of the units processed, the slowest rank's time, and per-unit
results gathered on rank 0, over whatever process group the caller made (gloo on CPU, NCCL on
GPUs).
"""
import numpy as np


def partition(weights, parts):
    """Longest-processing-time bin packing: units in descending weight order (ties by index) each
    go to the part with the least load so far (ties to the lowest part).  Returns one ascending
    index list per part; the same on every rank for the same weights."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    w = np.asarray(weights, dtype=np.float64)
    if w.ndim != 1 or np.any(w < 0) or not np.all(np.isfinite(w)):
        raise ValueError("weights must be finite and non-negative")
    order = sorted(range(len(w)), key=lambda i: (-w[i], i))
    load = [0.0] * parts
    out = [[] for _ in range(parts)]
    for i in order:
        p = min(range(parts), key=lambda q: (load[q], q))
        out[p].append(i)
        load[p] += float(w[i])
    return [sorted(x) for x in out]


def share(items, weights, rank, world):
    """The units of `items` that rank `rank` of `world` runs."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return [items[i] for i in partition(weights, world)[rank]]


def job_weight(desc, epochs):
    """Work of a served job: synapse slots times simulated seconds."""
    return float(desc.n_neurons) * float(desc.max_syn_per_neuron) * float(epochs) * \
        float(desc.epoch_duration)


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def reduce_timing(units, seconds, device=None):
    """Whole-job figures of an N-rank run: (sum of units, max of seconds) over the ranks; the
    local values when no process group is initialised.  device: where the reduction tensors live
    (a CUDA device for NCCL, None for gloo)."""
    dist = _dist()
    if dist is None:
        return float(units), float(seconds)
    import torch
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(u.item()), float(s.item())


def barrier():
    """All ranks meet (nothing without a group)."""
    dist = _dist()
    if dist is not None:
        dist.barrier()


def gather(obj):
    """Every rank's obj, in rank order, on rank 0 (None elsewhere); [obj] without a group."""
    dist = _dist()
    if dist is None:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out if dist.get_rank() == 0 else None


def latency_percentiles(latencies):
    """p50 / p95 / p99 of a list of job latencies (seconds), numpy's linear interpolation."""
    a = np.asarray(latencies, dtype=np.float64)
    if a.size == 0:
        return {"p50": None, "p95": None, "p99": None}
    return {"p50": float(np.percentile(a, 50)), "p95": float(np.percentile(a, 95)),
            "p99": float(np.percentile(a, 99))}
