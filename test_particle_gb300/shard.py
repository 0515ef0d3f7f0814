"""Particle sharding across GPUs (one process per GPU).

Particles are independent for the whole run (src/tracking.c:313,333) and the
fields are read-only, so each rank tracks a contiguous block of particles on
its own GPU with a replica of the field; the only exchange is one sum of the
diagnostics at the end, which the reference does with MPI_Reduce
(src/diagnostics.c:235,743-760).  These helpers restate that decomposition
for callers that use torch.distributed instead of MPI."""
import numpy as np


def shard_counts(nptl_tot, world):
    """Particles per rank: nptl_tot / world, the first nptl_tot % world ranks
    one more (particle_broadcast, src/particle_info.c:60-85)."""
    if world < 1 or nptl_tot < 0:
        raise ValueError("bad decomposition: %d particles over %d ranks" % (nptl_tot, world))
    return [nptl_tot // world + (1 if r < nptl_tot % world else 0) for r in range(world)]


def shard_range(nptl_tot, rank, world):
    """[start, stop) of this rank's particles."""
    c = shard_counts(nptl_tot, world)
    if not 0 <= rank < world:
        raise ValueError("rank %d outside 0..%d" % (rank, world - 1))
    start = int(sum(c[:rank]))
    return start, start + c[rank]


_SUMMED = ("espect", "espect_escape", "dsum", "remain")


def reduce_diagnostics(result, dist, group=None):
    """Sum the per-rank diagnostics (spectra counts, diffusion sums, particles
    remaining) over all ranks, in place, as the reference's MPI_Reduce does.
    `result` is the dict returned by track(); `dist` is torch.distributed.
    Counts are integers and stay exact; diffusion sums are added in rank order
    on every rank (all_reduce), so all ranks hold the same values."""
    import torch
    world = dist.get_world_size(group)
    for k in _SUMMED:
        a = np.ascontiguousarray(result[k])
        t = torch.from_numpy(a.astype(np.float64 if a.dtype.kind == "f" else np.int64))
        parts = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(parts, t, group=group)
        acc = parts[0].clone()
        for p in parts[1:]:
            acc += p
        result[k] = acc.numpy().astype(a.dtype).reshape(a.shape)
    return result
