"""Luminosity cache on the GPU: the first init computes the table and writes
the file, the next reads it (bit-identical table and cross section), a
corrupted file is recomputed and rewritten, a lock left by a dead process is
cleared, and polarized tables round-trip as two tables."""
import os
import subprocess
import sys

import numpy as np
import pytest

from upcgen_gb300 import lumi_cache as lc

pytestmark = pytest.mark.gpu

C1 = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "PROC_ID": 13, "FLUX_POINT": 1, "BREAKUP_MODE": 2, "MMIN": 3.56, "MMAX": 50,
      "BINS_M": 61, "YMIN": -6, "YMAX": 6, "BINS_Y": 31, "SEED": 1}


def _gen(ug, params, d, method=None):
    g = ug.UpcGenerator(params)
    g.setLumiFileDirectory(str(d))
    g.setLumiCache(True)
    if method is not None:
        g.setLumiMethod(method)
    g.init()
    return g


@pytest.mark.parametrize("method", ["plain", "fast"])
def test_write_then_read(ug, tmp_path, method):
    g1 = _gen(ug, C1, tmp_path, method)
    path, hit = g1.lumiCacheFile()
    assert hit == 0 and os.path.exists(path) and not os.path.exists(path + ".lock")
    lumi1 = g1.lumiTable()
    f = lc.read_lumi_cache(path)
    assert np.array_equal(f["tables"][0], lumi1)
    assert f["m"] == (3.56, 50.0, 61) and f["y"] == (-6.0, 6.0, 31)
    n0 = ug.kernel_launches()
    g2 = _gen(ug, C1, tmp_path, method)
    assert g2.lumiCacheFile() == (path, 1)
    assert np.array_equal(g2.lumiTable(), lumi1)
    assert g2.totNuclX() == g1.totNuclX()
    assert g2.timings()["lumi_ms"] < 50
    # the nuclear tables of a cache-hit init are complete when it returns
    # (the fast form builds G_AA beside the luminosity step it skipped)
    b = np.linspace(0.0, 20.0, 401)
    assert np.array_equal(g2.nucProcessCS.spline("gaa", b), g1.nucProcessCS.spline("gaa", b))
    assert np.array_equal(g2.nucProcessCS.spline("breakup", b), g1.nucProcessCS.spline("breakup", b))
    # the same events from the same table
    a, _ = g1.generateEvents(5000)
    b, _ = g2.generateEvents(5000)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    assert ug.kernel_launches() > n0
    # another configuration: another file, computed
    g3 = _gen(ug, dict(C1, BREAKUP_MODE=3), tmp_path, method)
    p3, hit3 = g3.lumiCacheFile()
    assert p3 != path and hit3 == 0 and os.path.exists(p3)


def test_corrupted_file_is_recomputed(ug, tmp_path):
    g1 = _gen(ug, C1, tmp_path)
    path, _ = g1.lumiCacheFile()
    raw = bytearray(open(path, "rb").read())
    raw[-100] ^= 0x40  # one payload bit
    open(path, "wb").write(bytes(raw))
    g2 = _gen(ug, C1, tmp_path)
    assert g2.lumiCacheFile()[1] == 0
    assert np.array_equal(g2.lumiTable(), g1.lumiTable())
    assert np.array_equal(lc.read_lumi_cache(path)["tables"][0], g1.lumiTable())
    # truncated
    open(path, "wb").write(bytes(raw[:200]))
    assert _gen(ug, C1, tmp_path).lumiCacheFile()[1] == 0
    assert _gen(ug, C1, tmp_path).lumiCacheFile()[1] == 1


def test_stale_lock_is_cleared(ug, tmp_path):
    path = ug.UpcGenerator(dict(C1))
    path.setLumiFileDirectory(str(tmp_path))
    fname, _ = path.lumiCacheFile()
    # a lock whose owner has exited
    p = subprocess.Popen([sys.executable, "-c", "pass"])
    p.wait()
    with open(fname + ".lock", "w") as f:
        f.write(f"{p.pid}\n")
    g = _gen(ug, C1, tmp_path)
    assert g.lumiCacheFile()[1] == 0
    assert os.path.exists(fname) and not os.path.exists(fname + ".lock")


def test_polarized_tables(ug, tmp_path):
    p = dict(C1, USE_POLARIZED_CS=1, BINS_M=21, BINS_Y=11)
    g1 = _gen(ug, p, tmp_path)
    s, ps = g1.lumiTable(polarized=True)
    path, hit = g1.lumiCacheFile()
    assert hit == 0
    t = lc.read_lumi_cache(path)["tables"]
    assert t.shape == (2, 21, 11) and np.array_equal(t[0], s) and np.array_equal(t[1], ps)
    g2 = _gen(ug, p, tmp_path)
    assert g2.lumiCacheFile()[1] == 1
    s2, ps2 = g2.lumiTable(polarized=True)
    assert np.array_equal(s2, s) and np.array_equal(ps2, ps)
    assert g2.totNuclX() == g1.totNuclX()


def test_cache_off_by_default(ug, tmp_path):
    g = ug.UpcGenerator(dict(C1, BINS_M=11, BINS_Y=7))
    g.setLumiFileDirectory(str(tmp_path))
    g.init()
    assert g.lumiCacheFile()[1] == -1
    assert os.listdir(tmp_path) == []


def test_lock_of_another_host(ug, tmp_path, monkeypatch):
    """A lock written by a process of another host (a shared luminosity
    directory) cannot be checked from here: it is left alone, and at the end
    of the wait the generator computes the table without writing the file."""
    monkeypatch.setenv("UPCG_LUMI_LOCK_TIMEOUT", "0.3")
    probe = ug.UpcGenerator(dict(C1))
    probe.setLumiFileDirectory(str(tmp_path))
    fname, _ = probe.lumiCacheFile()
    with open(fname + ".lock", "w") as f:
        f.write("some-other-host 1\n")
    g = _gen(ug, C1, tmp_path)
    assert g.lumiCacheFile()[1] == 0
    assert not os.path.exists(fname)
    assert open(fname + ".lock").read() == "some-other-host 1\n"
    os.unlink(fname + ".lock")
    g2 = _gen(ug, C1, tmp_path)
    assert np.array_equal(g2.lumiTable(), g.lumiTable())
    assert os.path.exists(fname) and not os.path.exists(fname + ".lock")
