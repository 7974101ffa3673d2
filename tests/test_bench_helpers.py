"""Host-side pieces of bench.py, on the CPU: the CPU sample's m-row blocks,
the batched-scan configurations, the workload name both arms print, and the
full-grid parity block computed on the committed fixture."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("nm,nblocks,block", [(1001, 4, 8), (1001, 8, 16), (201, 4, 8), (30, 4, 8)])
def test_row_blocks_inside_the_grid_and_disjoint(nm, nblocks, block):
    blocks = bench.row_blocks(nm, nblocks, block)
    assert blocks[0][0] == 0 and blocks[-1][1] == nm  # the lowest and the highest masses
    for a, b in blocks:
        assert 0 <= a < b <= nm
    for (a0, b0), (a1, b1) in zip(blocks, blocks[1:]):
        assert b0 <= a1
    if nblocks * block < nm:
        assert len(blocks) == nblocks and all(b - a == block for a, b in blocks)
    else:
        assert blocks == [(0, nm)]


def test_c5_configurations():
    cfg = bench.c5_configs()
    assert len(cfg) == 64
    assert {(c["NUCLEUS_Z"], c["NUCLEUS_A"]) for c in cfg} == {(82, 208), (79, 197), (54, 129), (8, 16)}
    assert {c["SQRTS"] for c in cfg} == {200, 5020, 5360, 5440}
    assert {c["BREAKUP_MODE"] for c in cfg} == {1, 2, 3, 4}
    assert {c["BINS_M"] for c in cfg} == {201, 501, 1001} and {c["BINS_Y"] for c in cfg} == {121}
    assert all(c["PROC_ID"] == 51 and c["ALP_MASS"] == 1 and c["ALP_WIDTH"] == 0.01 for c in cfg)


def test_workload_name_names_the_configuration():
    p = bench.WORKLOADS["c2"]
    s = bench.workload_name("c2", p, 1001, 121, bench.EVENTS["c2"])
    for part in ("1001x121", "FLUX_POINT 0", "BREAKUP_MODE 2", "PROC_ID 15", "10000000 events"):
        assert part in s, (part, s)


def test_parity_block_on_the_fixture():
    d = np.load(os.path.join(ROOT, "tests", "golden", "c2_lumi.npz"))
    conv, ref = d["conv"], d["ref"]
    # a table equal to the converged one: no error against it, and the
    # reference quadrature's own distance reported against the reference
    res = bench.c2_parity(conv.copy(), float(d["sigma_tot_conv"]), plain=ref.copy())
    fc = res["fast_vs_converged"]
    assert fc["all"]["cells"] == conv.size and fc["all"]["max_rel"] == 0.0
    assert res["fast_sigma_tot_vs_converged"] == 0.0
    assert res["plain_vs_reference_quadrature_max_rel"] == 0.0
    rq = res["reference_quadrature_vs_converged"]["above_1e-5_of_max"]
    assert rq["cells"] == 73324 and rq["cells_rel_above_1e-4"] == 142
    assert res["fast_vs_reference_quadrature"]["above_1e-5_of_max"]["cells_rel_above_1e-4"] == 142
    # a planted error of 2e-4 on one cell above 1e-4 of the maximum is counted
    bad = conv.copy()
    i = np.unravel_index(np.argmax(conv), conv.shape)
    bad[i] *= 1 + 2e-4
    res = bench.c2_parity(bad, float(d["sigma_tot_conv"]))
    assert res["fast_vs_converged"]["above_1e-4_of_max"]["cells_rel_above_1e-4"] == 1
