"""Event output on the host (no GPU): the HepMC3 text of records against a
restatement of the reference's WriterHepMC and writeEvent
(include/UpcGenerator.h:192-242, src/UpcGenerator.cpp:589-628), the particle
lists of generateEvent (:767-812), and the ROOT tree macro against stand-in
TFile / TTree headers."""
import os
import struct
import subprocess

import numpy as np
import pytest

from upcgen_gb300 import event_output as eo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _records(ug, n, seed):
    rng = np.random.default_rng(seed)
    ev = np.zeros(n, dtype=ug.EVENT_DTYPE)
    ev["m"] = rng.uniform(4, 50, n)
    ev["y"] = rng.uniform(-6, 6, n)
    ev["z"] = rng.uniform(-1, 1, n)
    ev["sign"] = rng.choice([-1.0, 1.0], n)
    for k in ("p0", "p1"):
        p = rng.normal(0, 10, (n, 3)) * np.exp(rng.uniform(-8, 8, (n, 1)))
        ev[k][:, :3] = p
        ev[k][:, 3] = np.sqrt((p.astype(np.float32).astype(np.float64) ** 2).sum(1) + 0.011)
    ev["p0"][0, 0] = -0.0  # negative zero prints as "-0"
    return ev


def _particles(e, pdg, charged, dpdg=0):
    """generateEvent's vectors for one record: (pdgs, statuses, mothers, momenta)."""
    a = [float(x) for x in e["p0"]]
    b = [float(x) for x in e["p1"]]
    if pdg == 51:
        return ([51, 22, 22], [23, 33, 33], [0, 1, 1],
                [[a[i] + b[i] for i in range(4)], a, b])
    if dpdg:  # vector meson: twoPartDecayVM's signed daughters
        s1 = 1 if e["sign"] > 0 else -1
        return ([pdg, s1 * dpdg, -s1 * dpdg], [23, 33, 33], [0, 1, 1],
                [[a[i] + b[i] for i in range(4)], a, b])
    s1 = (1 if e["sign"] > 0 else -1) if charged else 1
    s2 = -s1 if charged else 1
    return [s1 * pdg, s2 * pdg], [23, 23], [0, 0], [a, b]


def _mass(p):
    mm = p[3] * p[3] - (p[0] * p[0] + p[1] * p[1] + p[2] * p[2])
    return -np.sqrt(-mm) if mm < 0 else np.sqrt(mm)


def _hepmc_reference(events, pdg, charged, first, dpdg=0):
    out = []
    for i, e in enumerate(events):
        pdgs, sts, mos, ps = _particles(e, pdg, charged, dpdg)
        nv, last = -1, -1  # writeEvent's vertex count
        for m in mos:
            if m != last:
                nv += 1
                last = m
        out.append(f"E {first + i} {nv} {len(ps)}\nU GEV MM\n")
        for j, p in enumerate(ps):
            out.append("P %d %d %d %.9g %.9g %.9g %.9g %.9g %d\n"
                       % (j + 1, mos[j], pdgs[j], p[0], p[1], p[2], p[3], _mass(p), sts[j]))
    return "".join(out)


@pytest.mark.parametrize("proc,pdg,ppe,dpdg", [(13, 13, 2, 0), (15, 15, 2, 0), (51, 51, 3, 0),
                                               (443, 443, 3, 13), (553, 553, 3, 2212)])
def test_hepmc_text_matches_reference_writer(ug, proc, pdg, ppe, dpdg):
    g = ug.UpcGenerator({"PROC_ID": proc, "DECAY_PDG": dpdg})
    assert g.particlesPerEvent() == ppe
    assert g.decayPDG() == (dpdg or (22 if proc == 51 else 0))
    ev = _records(ug, 20000, proc)
    text = g.formatHepMC3(ev, first_event=17)
    assert text == _hepmc_reference(ev, pdg, True, 17, dpdg)
    events, rows = eo.read_hepmc3(text)
    assert len(events) == 20000 and events[0] == (17, 1 if ppe == 3 else 0, ppe)
    # 9 significant digits give back every float32 momentum exactly
    px = rows[:, 3].reshape(-1, ppe)
    col = 1 if ppe == 3 else 0
    assert np.array_equal(px[:, col].astype(np.float32), ev["p0"][:, 0])
    assert g.formatHepMC3(ev[:0]) == ""


def _write_columns(path, cols):
    n = len(cols["eventNumber"])
    hdr = b"UPCGPRT1" + struct.pack("=2IQ", 1, 9, n)
    for c in eo.COLUMNS:
        hdr += c.encode().ljust(16, b"\0") + (b"I" if c in eo.COLUMNS[:5] else b"D") + b"\0" * 7
    body = b""
    for c in eo.COLUMNS:
        a = np.ascontiguousarray(cols[c], dtype=np.int32 if c in eo.COLUMNS[:5] else np.float64).tobytes()
        body += a + b"\0" * ((len(a) + 7) // 8 * 8 - len(a))
    open(path, "wb").write(hdr + body)


_TFILE = r"""#pragma once
#include <cstdio>
struct TFile {
  static FILE*& out() { static FILE* f = nullptr; return f; }
  TFile(const char* name, const char*) { out() = std::fopen(name, "w"); }
  void Close() { if (out()) std::fclose(out()); out() = nullptr; }
};
"""
_TTREE = r"""#pragma once
#include <cstdio>
#include <string>
#include <vector>
#include "TFile.h"
struct TTree {
  struct B { std::string name, leaf; void* p; };
  std::vector<B> br; long entries = 0;
  TTree(const char* n, const char*) { std::fprintf(TFile::out(), "tree %s\n", n); }
  void Branch(const char* n, void* p, const char* leaf) { br.push_back({n, leaf, p}); }
  void Fill() {
    for (auto& b : br) {
      if (b.leaf.back() == 'I') std::fprintf(TFile::out(), "%d ", *static_cast<int*>(b.p));
      else std::fprintf(TFile::out(), "%a ", *static_cast<double*>(b.p));
    }
    std::fprintf(TFile::out(), "\n");
    ++entries;
  }
  void Write() {
    for (auto& b : br) std::fprintf(TFile::out(), "branch %s %s\n", b.name.c_str(), b.leaf.c_str());
  }
};
"""
_MAIN = r"""int particles_to_root(const char*, const char*);
int main(int, char** v) { return particles_to_root(v[1], v[2]); }
"""


def test_vector_meson_configuration_errors(ug):
    # src/UpcPhotoNuclearVM.cpp:80-87: the decay mode must be one the meson knows
    with pytest.raises(ug.UpcgError, match="DECAY_PDG"):
        ug.UpcGenerator({"PROC_ID": 443}).particlesPerEvent()
    with pytest.raises(ug.UpcgError, match="SHADOWING"):
        ug.UpcGenerator({"PROC_ID": 443, "DECAY_PDG": 13, "SHADOWING": 2}).particlesPerEvent()
    # the generator's single mass bin around m_V (src/UpcGenerator.cpp:131-140)
    g = ug.UpcGenerator({"PROC_ID": 553, "DECAY_PDG": 11, "BINS_M": 50})
    g.particlesPerEvent()
    gr = g.grid()
    assert gr["nm"] == 1 and abs(gr["mmin"] - (9.3987 - 1e-6)) < 1e-12


def test_particles_root_macro(tmp_path):
    for name, text in (("TFile.h", _TFILE), ("TTree.h", _TTREE), ("main.cpp", _MAIN)):
        (tmp_path / name).write_text(text)
    exe = tmp_path / "conv"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(tmp_path), str(tmp_path / "main.cpp"),
                    os.path.join(ROOT, "upcgen_gb300", "particles_to_root.C"), "-o", str(exe)],
                   check=True)
    rng = np.random.default_rng(1)
    n = 7  # odd: int columns need padding
    cols = {c: rng.integers(-50, 50, n) for c in eo.COLUMNS[:5]}
    cols.update({c: rng.normal(size=n) for c in eo.COLUMNS[5:]})
    _write_columns(tmp_path / "ev.cols", cols)
    r = eo.read_particle_columns(tmp_path / "ev.cols")
    assert all(np.array_equal(r[c], cols[c]) for c in eo.COLUMNS)
    subprocess.run([str(exe), str(tmp_path / "ev.cols"), str(tmp_path / "out.txt")], check=True)
    lines = (tmp_path / "out.txt").read_text().strip().split("\n")
    assert lines[0] == "tree particles"
    assert lines[-9:] == [f"branch {c} {c}/{'I' if c in eo.COLUMNS[:5] else 'D'}" for c in eo.COLUMNS]
    for r_, line in enumerate(lines[1:1 + n]):
        v = line.split()
        assert [int(x) for x in v[:5]] == [int(cols[c][r_]) for c in eo.COLUMNS[:5]]
        assert [float.fromhex(x) for x in v[5:]] == [float(cols[c][r_]) for c in eo.COLUMNS[5:]]


@pytest.mark.parametrize("proc,dpdg", [(13, 0), (15, 0), (51, 0), (443, 13), (553, 2212)])
def test_particle_lists(ug, proc, dpdg):
    """particlesOf / getParticles against the restatement of generateEvent's
    lists above and against the HepMC3 text of the same records."""
    g = ug.UpcGenerator({"PROC_ID": proc, "DECAY_PDG": dpdg})
    assert g.getParticles() == []
    ev = _records(ug, 300, proc + 1)
    events, rows = eo.read_hepmc3(g.formatHepMC3(ev))
    ppe = g.particlesPerEvent()
    pdg = 51 if proc == 51 else proc
    for k, e in enumerate(ev):
        got = g.particlesOf(e)
        pdgs, sts, mos, ps = _particles(e, pdg, True, dpdg)
        assert [p[0] for p in got] == pdgs
        assert [p[1] for p in got] == sts and [p[2] for p in got] == mos
        assert all(tuple(q) == tuple(r) for (_, _, _, q), r in zip(got, ps))
        assert [int(x) for x in rows[k * ppe:(k + 1) * ppe, 2]] == pdgs


def _ref_hepmc():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_ref_hepmc
    return make_ref_hepmc


@pytest.mark.parametrize("name", ["mumu", "tautau", "alp"])
def test_hepmc_text_is_the_reference_writers(ug, name):
    """The library's HepMC3 text against the reference's own writeEvent and
    WriterHepMC (src/UpcGenerator.cpp:589-628, include/UpcGenerator.h:192-242),
    compiled from its sources (tests/golden/make_ref_hepmc.py): for seeded
    records, the reference's file of the library's particle lists is the
    library's preamble + formatHepMC3 + end line, byte for byte (SHA-256 and
    size committed in tests/golden/ref_hepmc.json; compared directly when the
    reference sources are present).  tests/test_gpu_event_output.py checks
    that the library's files are that preamble + formatHepMC3 + end line."""
    import hashlib
    import json
    mk = _ref_hepmc()
    from test_gpu_event_output import HEAD, TAIL
    with open(os.path.join(os.path.dirname(__file__), "golden", "ref_hepmc.json")) as f:
        want = json.load(f)[name]
    proc, n, seed, first = mk.CASES[name]
    assert (want["proc"], want["records"], want["seed"], want["first_event"]) == (proc, n, seed, first)
    g = ug.UpcGenerator({"PROC_ID": proc})
    ev = mk.records(ug.EVENT_DTYPE, n, seed)
    ours = (HEAD + g.formatHepMC3(ev, first_event=first) + TAIL).encode()
    assert len(ours) == want["bytes"]
    assert hashlib.sha256(ours).hexdigest() == want["sha256"]
    from oracle import build as ob
    if ob.build_ref_gen() is not None:
        assert mk.reference_text(*mk.particle_arrays(g, ev), first) == ours


@pytest.mark.parametrize("proc,pdg", [(13, 13), (51, 51)])
def test_hepmc_text_extreme_values(ug, proc, pdg):
    """The %.9g text of every kind of FP32 momentum -- random bit patterns
    over all exponents, subnormals, +-0, the largest floats -- and of the
    masses and sums formed from them in FP64, against Python's correctly
    rounded '%.9g' of the same values."""
    g = ug.UpcGenerator({"PROC_ID": proc})
    rng = np.random.default_rng(2024)
    n = 20000
    bits = rng.integers(0, 2 ** 32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
    vals = bits.view(np.float32)
    vals[~np.isfinite(vals)] = 1.0
    special = np.array([0.0, -0.0, 1e-45, -1e-45, 1.1754942e-38, 3.4028235e38, -3.4028235e38,
                        0.1, 1e-10, 123456789.0, 999999999.0, 1e9, 9.99999999e-5], dtype=np.float32)
    vals[: len(special), 0] = special
    ev = np.zeros(n, dtype=ug.EVENT_DTYPE)
    ev["sign"] = rng.choice([-1.0, 1.0], n)
    ev["p0"], ev["p1"] = vals[:, :4], vals[:, 4:]
    text = g.formatHepMC3(ev, first_event=3)
    assert text == _hepmc_reference(ev, pdg, True, 3)
