"""Sharding of the luminosity / sampling path over ranks (one GPU per rank).

The luminosity cells are independent, as in the reference's OpenMP m-slices
(src/UpcCrossSection.cpp:537-538): rank r computes the contiguous m-rows
``row_range(nm, r, world)``, the row blocks are all-gathered into the full
table, and every rank builds the (replicated) cross section and samplers from
it.  Events need no exchange: rank r draws candidates from its own Philox
counter range starting at ``candidate_offset(r)``.

The functions take a ``torch.distributed`` process group (NCCL on GPUs, gloo
on host ranks) or ``None`` for a single process.  With NCCL the rows never
leave the GPU: the library's device table is viewed in place, all-gathered
device to device, and installed from device memory
(``upcg_set_lumi_table_device``).  With gloo the rows travel through host
memory.  Polarized configurations (USE_POLARIZED_CS, the ALP) gather the
scalar and the pseudoscalar tables.
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


def _max_rows(nm, world):
    return max(row_range(nm, r, world)[1] - row_range(nm, r, world)[0] for r in range(world))


def gather_rows(local_rows, nm, rank, world, group=None):
    """All-gather the row blocks [im0, im1) x ny of every rank into the full
    (nm, ny) table through host memory (FP64, bit-exact: the blocks travel as
    raw doubles).  For host ranks (gloo); GPU ranks use gather_rows_device."""
    local_rows = np.ascontiguousarray(local_rows, dtype=np.float64)
    ny = local_rows.shape[1]
    if world == 1:
        return local_rows.copy()
    import torch
    import torch.distributed as dist
    pad = torch.zeros((_max_rows(nm, world), ny), dtype=torch.float64)
    pad[: local_rows.shape[0]] = torch.from_numpy(local_rows)
    bufs = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    out = np.empty((nm, ny), dtype=np.float64)
    for r in range(world):
        a, b = row_range(nm, r, world)
        out[a:b] = bufs[r][: b - a].numpy()
    return out


def gather_rows_device(local_rows, nm, rank, world, group=None):
    """All-gather device row blocks (a CUDA float64 tensor [im1 - im0][ny])
    into a contiguous device table [nm][ny] over NCCL; nothing passes
    through host memory."""
    import torch
    import torch.distributed as dist
    ny = local_rows.shape[1]
    pad = torch.zeros((_max_rows(nm, world), ny), dtype=torch.float64, device=local_rows.device)
    pad[: local_rows.shape[0]].copy_(local_rows)
    bufs = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    parts = []
    for r in range(world):
        a, b = row_range(nm, r, world)
        parts.append(bufs[r][: b - a])
    return torch.cat(parts).contiguous()


class _DeviceTable:
    """A view of the library's device table for torch (__cuda_array_interface__;
    no copy)."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}


def sharded_init(gen, rank, world, group=None):
    """Luminosity rows of this rank, all-gathered, installed; samplers built;
    the event sequence moved to this rank's counter range.  Returns the full
    luminosity table(s): device tensors with NCCL, numpy arrays otherwise
    (a tuple (scalar, pseudoscalar) when polarized)."""
    g = gen.grid()
    nm, ny = g["nm"], g["ny"]
    im0, im1 = row_range(nm, rank, world)
    gen.setRowRange(im0, im1)
    gen.init()  # returns with the rows complete on the device
    ptr, ptr2 = gen.lumiTableDevicePtrs()
    polarized = bool(ptr2)
    if world == 1:
        gen.setCandidateOffset(candidate_offset(rank))
        return gen.lumiTable(polarized=polarized)
    import torch.distributed as dist
    if dist.get_backend(group) == "nccl":
        import torch
        views = [torch.as_tensor(_DeviceTable(p, (nm, ny)), device="cuda")
                 for p in ((ptr, ptr2) if polarized else (ptr,))]
        fulls = [gather_rows_device(v[im0:im1], nm, rank, world, group) for v in views]
        torch.cuda.current_stream().synchronize()  # the gather is complete
        n = nm * ny
        gen.setLumiTableDevice(fulls[0].data_ptr(), n, fulls[1].data_ptr() if polarized else None)
    else:
        tabs = gen.lumiTable(polarized=True) if polarized else (gen.lumiTable(),)
        fulls = [gather_rows(t[im0:im1], nm, rank, world, group) for t in tabs]
        gen.setLumiTable(fulls[0], fulls[1] if polarized else None)
    gen.setCandidateOffset(candidate_offset(rank))
    return tuple(fulls) if polarized else fulls[0]
