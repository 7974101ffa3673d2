"""upcg_flux_form_device_noalloc (no counterpart in the reference): fluxForm on
device buffers with its QAGS scratch in static device memory.

Collected last on purpose: it must pass on its own and after every other GPU
test in the same process.  It checks the no-allocation entry against the
allocating upcg_flux_form on two calls in a row, that device free memory does
not move across those calls (after the first call, which does the set-up),
and the documented size / state errors.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PB_FORM = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
           "PROC_ID": 15, "LEP_A": 0, "FLUX_POINT": 0, "BREAKUP_MODE": 2,
           "MMIN": 3.56, "MMAX": 50, "BINS_M": 3, "YMIN": -6, "YMAX": 6, "BINS_Y": 3}


def _points(rng, n):
    # b across the form-factor region and beyond 2R (the point-flux branch)
    b = np.exp(rng.uniform(np.log(0.3), np.log(40.0), n))
    k = np.exp(rng.uniform(np.log(0.01), np.log(300.0), n))
    return b, k


def test_noalloc_flux_form_matches_allocating_entry(ug):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    g = ug.UpcGenerator(PB_FORM)
    g.setStream(stream.cuda_stream)
    g.init()
    cs = g.nucProcessCS
    rng = np.random.default_rng(7)
    # first call: set-up (scratch address lookup)
    b, k = _points(rng, 64)
    db = torch.tensor(b, dtype=torch.float64, device="cuda")
    dk = torch.tensor(k, dtype=torch.float64, device="cuda")
    dout = torch.empty_like(db)
    torch.cuda.synchronize()
    cs.fluxFormDeviceNoAlloc(db.data_ptr(), dk.data_ptr(), dout.data_ptr(), b.size)
    stream.synchronize()
    # two calls in a row on fresh inputs, device buffers made beforehand
    n = 3000
    pts = [_points(rng, n) for _ in range(2)]
    bufs = []
    for b, k in pts:
        bufs.append((torch.tensor(b, dtype=torch.float64, device="cuda"),
                     torch.tensor(k, dtype=torch.float64, device="cuda"),
                     torch.full((n,), float("nan"), dtype=torch.float64, device="cuda"),
                     torch.full((1,), -1, dtype=torch.int32, device="cuda")))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for db, dk, dout, dfail in bufs:
        cs.fluxFormDeviceNoAlloc(db.data_ptr(), dk.data_ptr(), dout.data_ptr(), n,
                                 dfail.data_ptr())
    stream.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    for (b, k), (db, dk, dout, dfail) in zip(pts, bufs):
        ref = cs.fluxForm(b, k)
        failures_ref = g.qagsStats()["failures"]
        out = dout.cpu().numpy()
        # the same kernel on the same points: bit-identical
        assert np.array_equal(out, ref), np.max(np.abs(out - ref) / np.abs(ref))
        assert int(dfail.item()) == failures_ref


def test_noalloc_errors(ug):
    g = ug.UpcGenerator(PB_FORM)
    one = ug.np.zeros(1)
    # before upcg_init: no tables, nothing launched
    with pytest.raises(ug.UpcgError, match="needs the tables"):
        g.nucProcessCS.fluxFormDeviceNoAlloc(one.ctypes.data, one.ctypes.data, one.ctypes.data, 1)
    # beyond the stated maximum: rejected before any device work
    with pytest.raises(ug.UpcgError, match="at most"):
        g.nucProcessCS.fluxFormDeviceNoAlloc(one.ctypes.data, one.ctypes.data, one.ctypes.data,
                                             16777216 + 1)
