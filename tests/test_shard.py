"""Host-side sharding of the luminosity over ranks (upcgen_gb300.shard), run
as gloo ranks on the CPU: each rank computes its m-rows with the oracle (the
GPU part is covered by tests/test_gpu_shard.py), the rows are all-gathered,
and the gathered table must equal the single-process table bit for bit."""
import os
import socket

import numpy as np
import pytest

from upcgen_gb300 import shard

SMALL = {"PROC_ID": 13, "FLUX_POINT": 1, "BREAKUP_MODE": 2, "MMIN": 3.56, "MMAX": 20,
         "BINS_M": 7, "YMIN": -3, "YMAX": 3, "BINS_Y": 5}


@pytest.mark.parametrize("nm,world", [(7, 2), (1001, 3), (201, 8), (3, 3), (5, 1)])
def test_row_ranges_cover_the_grid(nm, world):
    rr = [shard.row_range(nm, r, world) for r in range(world)]
    assert rr[0][0] == 0 and rr[-1][1] == nm
    assert all(rr[i][1] == rr[i + 1][0] for i in range(world - 1))
    sizes = [b - a for a, b in rr]
    assert max(sizes) - min(sizes) <= 1


def test_candidate_ranges_disjoint():
    offs = [shard.candidate_offset(r) for r in range(8)]
    assert all(b - a == shard.COUNTER_STRIDE for a, b in zip(offs, offs[1:]))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import Oracle
    o = Oracle(SMALL, threads=1)
    o.init_tables()
    nm = o.grid()["nm"]
    im0, im1 = shard.row_range(nm, rank, world)
    rows = o.lumi_table(im0, im1)
    full = shard.gather_rows(rows, nm, rank, world)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_gather_equals_single(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.oracle import Oracle
    out = str(tmp_path / "full.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn",
                       join=True)
    o = Oracle(SMALL, threads=1)
    o.init_tables()
    ref = o.lumi_table()
    got = np.load(out)
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


def _rank_main_pol(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import Oracle
    o = Oracle(dict(SMALL, USE_POLARIZED_CS=1), threads=1)
    o.init_tables()
    nm = o.grid()["nm"]
    im0, im1 = shard.row_range(nm, rank, world)
    s, p = o.lumi_table(im0, im1, polarized=True)
    full = [shard.gather_rows(t, nm, rank, world) for t in (s, p)]
    if rank == 0:
        np.save(out_path, np.stack(full))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_polarized_pair(tmp_path):
    """Polarized configurations shard both tables (scalar and pseudoscalar,
    calcTwoPhotonLumiPol, src/UpcCrossSection.cpp:274-335)."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.oracle import Oracle
    out = str(tmp_path / "pol.npy")
    mp.start_processes(_rank_main_pol, args=(2, _free_port(), out), nprocs=2, start_method="spawn",
                       join=True)
    o = Oracle(dict(SMALL, USE_POLARIZED_CS=1), threads=1)
    o.init_tables()
    s, p = o.lumi_table(polarized=True)
    got = np.load(out)
    assert np.array_equal(got[0], s) and np.array_equal(got[1], p)
