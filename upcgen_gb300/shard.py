"""Sharding of the luminosity / sampling path over ranks (one GPU per rank).

The luminosity cells are independent, as in the reference's OpenMP m-slices
(src/UpcCrossSection.cpp:537-538): rank r computes the contiguous m-rows
``row_range(nm, r, world)``, the row blocks are all-gathered into the full
table, and every rank builds the (replicated) cross section and samplers from
it.  Events need no exchange: rank r draws candidates from its own Philox
counter range starting at ``candidate_offset(r)``.

The functions take a ``torch.distributed`` process group (NCCL on GPUs, gloo
on host ranks) or ``None`` for a single process.
"""
import numpy as np

# Philox counters per rank: 2^48 candidates each, far beyond any run
COUNTER_STRIDE = 1 << 48


def row_range(nm, rank, world):
    """Contiguous m-rows [im0, im1) of rank `rank`: sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, extra = divmod(nm, world)
    im0 = rank * base + min(rank, extra)
    return im0, im0 + base + (1 if rank < extra else 0)


def candidate_offset(rank):
    return rank * COUNTER_STRIDE


def gather_rows(local_rows, nm, rank, world, group=None):
    """All-gather the row blocks [im0, im1) x ny of every rank into the full
    (nm, ny) table (FP64, bit-exact: the blocks travel as raw doubles)."""
    local_rows = np.ascontiguousarray(local_rows, dtype=np.float64)
    ny = local_rows.shape[1]
    if world == 1:
        return local_rows.copy()
    import torch
    import torch.distributed as dist
    maxr = max(row_range(nm, r, world)[1] - row_range(nm, r, world)[0] for r in range(world))
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    pad = torch.zeros((maxr, ny), dtype=torch.float64, device=dev)
    pad[: local_rows.shape[0]] = torch.from_numpy(local_rows).to(dev)
    bufs = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    out = np.empty((nm, ny), dtype=np.float64)
    for r in range(world):
        a, b = row_range(nm, r, world)
        out[a:b] = bufs[r][: b - a].cpu().numpy()
    return out


def sharded_init(gen, rank, world, group=None):
    """Luminosity rows of this rank, all-gathered, installed; samplers built;
    the event sequence moved to this rank's counter range.  Returns the full
    luminosity table."""
    nm = gen.grid()["nm"]
    im0, im1 = row_range(nm, rank, world)
    gen.setRowRange(im0, im1)
    gen.init()
    full = gather_rows(gen.lumiTable()[im0:im1], nm, rank, world, group)
    gen.setLumiTable(full)
    gen.setCandidateOffset(candidate_offset(rank))
    return full
