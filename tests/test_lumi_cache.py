"""Luminosity cache (host side, no GPU): the key names every input of the
table and nothing else, the file layout round-trips through the Python reader,
corruption is detected, and the ROOT export macro writes the reference's
histogram layout (src/UpcCrossSection.cpp:481-503, 556-585).  The GPU-side
write / read / recompute cycle is in test_gpu_lumi_cache.py."""
import os
import struct
import subprocess

import numpy as np
import pytest

from upcgen_gb300 import lumi_cache as lc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C1 = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "PROC_ID": 13, "FLUX_POINT": 1, "BREAKUP_MODE": 1, "MMIN": 3.56, "MMAX": 50,
      "BINS_M": 201, "YMIN": -6, "YMAX": 6, "BINS_Y": 61, "SEED": 1}


def _file(ug, params, method=None, directory=None):
    g = ug.UpcGenerator(params)
    if method is not None:
        g.setLumiMethod(method)
    if directory is not None:
        g.setLumiFileDirectory(directory)
    return g.lumiCacheFile()


def test_key_covers_table_inputs_only(ug, tmp_path):
    base, hit = _file(ug, C1)
    assert hit == -1
    assert os.path.basename(base).startswith("upcg_lumi_") and base.endswith(".bin")
    # inputs of the table: each changes the file
    for k, v in (("NUCLEUS_Z", 79), ("NUCLEUS_A", 197), ("WS_R", 6.38), ("WS_A", 0.535),
                 ("SQRTS", 5360), ("FLUX_POINT", 0), ("BREAKUP_MODE", 2), ("MMIN", 4.0),
                 ("MMAX", 40), ("BINS_M", 200), ("YMIN", -5), ("YMAX", 5), ("BINS_Y", 60),
                 ("USE_POLARIZED_CS", 1), ("WS_R", 6.68 * (1 + 2 ** -52))):
        assert _file(ug, dict(C1, **{k: v}))[0] != base, k
    assert _file(ug, C1, method="fast")[0] != base
    assert _file(ug, C1, method="grid")[0] != base
    # not inputs of the table: same file (tau pairs keep MMIN = 3.56 >= 2 m_tau)
    for k, v in (("SEED", 7), ("NEVENTS", 10), ("PROC_ID", 15), ("DO_PT_CUT", 1),
                 ("PT_MIN", 1.0), ("DO_ETA_CUT", 1), ("ETA_MIN", -2.4), ("BINS_Z", 50),
                 ("NON_ZERO_GAM_PT", 0)):
        assert _file(ug, dict(C1, **{k: v}))[0] == base, k
    # the directory
    d = str(tmp_path)
    assert _file(ug, C1, directory=d)[0] == os.path.join(d, os.path.basename(base))


def test_key_uses_derived_mass_range(ug):
    # ALP: the mass range is forced to M -+ 4 Gamma (src/UpcGenerator.cpp:105-115)
    alp = dict(C1, PROC_ID=51, ALP_MASS=1, ALP_WIDTH=0.01)
    assert _file(ug, alp)[0] == _file(ug, dict(alp, MMIN=2, MMAX=99))[0]


def _write(path, key, tables):
    """The documented layout, written independently of the library."""
    tables = np.ascontiguousarray(tables, dtype=np.float64)
    ntab, nm, ny = tables.shape
    kb = key.encode()
    pad = kb + b"\0" * ((len(kb) + 7) // 8 * 8 - len(kb))
    payload = tables.tobytes()
    with open(path, "wb") as f:
        f.write(lc.MAGIC + struct.pack("=4I", 1, ntab, nm, ny) + struct.pack("=Q", len(kb)) + pad +
                struct.pack("=Q", lc.fnv1a64(payload)) + payload)


KEY = ("upcgen_gb300 two-photon luminosity L dm dy [nm][ny]; revision 1; method 0; Z 82; "
       "A 208; R 0x1.ab851eb851eb8p+2; m [0x1.c7ae147ae147bp+1, 0x1.9p+5] bins 5; "
       "y [-0x1.8p+2, 0x1.8p+2] bins 3")


def test_reader_round_trip_and_corruption(tmp_path):
    rng = np.random.default_rng(3)
    t = rng.random((2, 5, 3))
    p = tmp_path / "c.bin"
    _write(p, KEY, t)
    r = lc.read_lumi_cache(p)
    assert np.array_equal(r["tables"], t) and r["key"] == KEY
    assert r["m"] == (3.56, 50.0, 5) and r["y"] == (-6.0, 6.0, 3)
    raw = bytearray(p.read_bytes())
    raw[-3] ^= 0x10
    p.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        lc.read_lumi_cache(p)
    p.write_bytes(bytes(raw[:-8]))
    with pytest.raises(ValueError, match="payload"):
        lc.read_lumi_cache(p)
    p.write_bytes(b"XXXXXXXX" + bytes(raw[8:]))
    with pytest.raises(ValueError, match="not a luminosity"):
        lc.read_lumi_cache(p)


# minimal stand-ins for ROOT's TFile / TH2D: record what the macro writes
_TFILE = r"""#pragma once
#include <cstdio>
struct TFile {
  static FILE*& out() { static FILE* f = nullptr; return f; }
  TFile(const char* name, const char*) { out() = std::fopen(name, "w"); }
  void Close() { if (out()) std::fclose(out()); out() = nullptr; }
};
"""
_TH2D = r"""#pragma once
#include <string>
#include <vector>
#include "TFile.h"
struct TH2D {
  std::string name; int nx, ny; double xlo, xhi, ylo, yhi; std::vector<double> c;
  TH2D(const char* n, const char*, int nx_, double xlo_, double xhi_, int ny_, double ylo_,
       double yhi_) : name(n), nx(nx_), ny(ny_), xlo(xlo_), xhi(xhi_), ylo(ylo_), yhi(yhi_),
                      c((nx_ + 2) * (ny_ + 2), 0.) {}
  void SetBinContent(int i, int j, double v) { c[j * (nx + 2) + i] = v; }
  void Write() {
    std::fprintf(TFile::out(), "%s %d %a %a %d %a %a\n", name.c_str(), nx, xlo, xhi, ny, ylo, yhi);
    for (int j = 0; j < ny + 2; ++j)
      for (int i = 0; i < nx + 2; ++i) std::fprintf(TFile::out(), "%a\n", c[j * (nx + 2) + i]);
  }
};
"""
_MAIN = r"""int lumi_cache_to_root(const char*, const char*);
int main(int, char** v) { return lumi_cache_to_root(v[1], v[2]); }
"""


@pytest.mark.parametrize("ntab", [1, 2])
def test_root_export_macro(tmp_path, ntab):
    (tmp_path / "TFile.h").write_text(_TFILE)
    (tmp_path / "TH2D.h").write_text(_TH2D)
    (tmp_path / "main.cpp").write_text(_MAIN)
    exe = tmp_path / "conv"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(tmp_path), str(tmp_path / "main.cpp"),
                    os.path.join(ROOT, "upcgen_gb300", "lumi_cache_to_root.C"), "-o", str(exe)],
                   check=True)
    t = np.random.default_rng(ntab).random((ntab, 5, 3))
    _write(tmp_path / "c.bin", KEY, t)
    out = tmp_path / "out.txt"
    subprocess.run([str(exe), str(tmp_path / "c.bin"), str(out)], check=True)
    lines = out.read_text().split("\n")
    names = ["hD2LDMDY"] if ntab == 1 else ["hD2LDMDY_s", "hD2LDMDY_p"]
    pos = 0
    for k, name in enumerate(names):
        hdr = lines[pos].split()
        assert hdr[0] == name and int(hdr[1]) == 5 and int(hdr[4]) == 3
        assert float.fromhex(hdr[2]) == 3.56 and float.fromhex(hdr[3]) == 50.0
        assert float.fromhex(hdr[5]) == -6.0 and float.fromhex(hdr[6]) == 6.0
        c = np.array([float.fromhex(x) for x in lines[pos + 1:pos + 1 + 7 * 5]]).reshape(5, 7)
        # bin (im + 1, iy + 1) = table[im][iy]; under/overflow empty
        assert np.array_equal(c[1:4, 1:6].T, t[k])
        assert not c[0].any() and not c[4].any() and not c[:, 0].any() and not c[:, 6].any()
        pos += 1 + 7 * 5
    # a corrupted file is refused
    raw = bytearray((tmp_path / "c.bin").read_bytes())
    raw[-1] ^= 1
    (tmp_path / "c.bin").write_bytes(bytes(raw))
    assert subprocess.run([str(exe), str(tmp_path / "c.bin"), str(out)]).returncode != 0
