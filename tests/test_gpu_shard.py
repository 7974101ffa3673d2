"""Sharded luminosity on one GPU: two generators compute the two m-row halves
(as two ranks would), the halves are joined and installed, and the result must
equal the single-handle tables bit for bit; disjoint candidate offsets give
disjoint event streams."""
import numpy as np
import pytest

from upcgen_gb300 import shard

pytestmark = pytest.mark.gpu

P = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
     "PROC_ID": 13, "FLUX_POINT": 1, "BREAKUP_MODE": 2, "MMIN": 3.56, "MMAX": 50,
     "BINS_M": 41, "YMIN": -6, "YMAX": 6, "BINS_Y": 25, "SEED": 3}


@pytest.mark.parametrize("method", ["plain", "fast"])
def test_two_shards_equal_one(ug, method):
    full = ug.UpcGenerator(P)
    full.setLumiMethod(method)
    full.init()
    ref = full.lumiTable()
    _, ref_tot = full.nucCSYM()
    nm = full.grid()["nm"]
    parts = []
    for r in range(2):
        g = ug.UpcGenerator(P)
        g.setLumiMethod(method)
        a, b = shard.row_range(nm, r, 2)
        g.setRowRange(a, b)
        g.init()
        t = g.lumiTable()
        assert not t[:a].any() and not t[b:].any()  # only its rows
        parts.append(t[a:b])
    joined = np.concatenate(parts)
    assert np.array_equal(joined, ref)
    g = ug.UpcGenerator(P)
    g.setLumiMethod(method)
    g.setLumiTable(joined)
    _, tot = g.nucCSYM()
    assert tot == ref_tot
    ev0, _ = g.generateEvents(1000)
    ev_ref, _ = full.generateEvents(1000)
    assert np.array_equal(ev0, ev_ref)  # offset 0: the same candidate stream
    g.setCandidateOffset(shard.candidate_offset(1))
    ev1, _ = g.generateEvents(1000)
    assert not np.array_equal(ev1["m"], ev0["m"])


@pytest.mark.parametrize("method", ["plain", "fast"])
def test_two_shards_polarized(ug, method):
    """USE_POLARIZED_CS: both tables are sharded, joined and installed; the
    cross section and its total equal the single-handle ones."""
    p = dict(P, USE_POLARIZED_CS=1, BINS_M=21, BINS_Y=13)
    full = ug.UpcGenerator(p)
    full.setLumiMethod(method)
    full.init()
    rs, rp = full.lumiTable(polarized=True)
    _, ref_tot = full.nucCSYM()
    nm = full.grid()["nm"]
    ps, pp = [], []
    for r in range(2):
        g = ug.UpcGenerator(p)
        g.setLumiMethod(method)
        a, b = shard.row_range(nm, r, 2)
        g.setRowRange(a, b)
        g.init()
        s, q = g.lumiTable(polarized=True)
        ps.append(s[a:b])
        pp.append(q[a:b])
    js, jp = np.concatenate(ps), np.concatenate(pp)
    assert np.array_equal(js, rs) and np.array_equal(jp, rp)
    g = ug.UpcGenerator(p)
    g.setLumiMethod(method)
    g.setLumiTable(js, jp)
    assert g.nucCSYM()[1] == ref_tot


def test_install_from_device_memory(ug):
    """upcg_set_lumi_table_device (the NCCL gather's install) gives what the
    host install gives; the device view of the library's table reads back
    the host table."""
    torch = pytest.importorskip("torch")
    full = ug.UpcGenerator(P)
    full.init()
    ref = full.lumiTable()
    ptr, ptr2 = full.lumiTableDevicePtrs()
    assert ptr2 == 0
    view = torch.as_tensor(shard._DeviceTable(ptr, ref.shape), device="cuda")
    assert np.array_equal(view.cpu().numpy(), ref)
    dev = view.clone()
    torch.cuda.synchronize()
    g = ug.UpcGenerator(P)
    g.setLumiTableDevice(dev.data_ptr(), ref.size)
    assert np.array_equal(g.lumiTable(), ref)
    assert g.nucCSYM()[1] == full.nucCSYM()[1]
    ev, _ = g.generateEvents(500)
    ev_ref, _ = full.generateEvents(500)
    assert np.array_equal(ev, ev_ref)
