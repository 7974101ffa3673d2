"""The C ABI library loads and exports every symbol include/upcgen_gb300.h
declares; configuration runs without a GPU (no compute calls here)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "upcgen_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(upcg_\w+)\s*\(", text, re.M)))


def test_every_declared_symbol_is_exported(ug):
    L = ug.load_library()
    syms = header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert sorted(ug.ABI_SYMBOLS) == syms


def test_sm103a_only(ug):
    from upcgen_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_config_file_parsing(ug, tmp_path):
    # src/UpcGenerator.cpp:318-346: '#' lines, trailing comments, unknown keys ignored
    p = tmp_path / "parameters.in"
    p.write_text("# a comment line\n"
                 "BINS_M 17   # trailing comment\n"
                 "BINS_Y 9\n"
                 "YMIN -2.5\n"
                 "PYTHIA_VERSION 8\n"
                 "SOME_UNKNOWN_KEY 42\n"
                 "\n"
                 "MMAX 20\n")
    g = ug.UpcGenerator()
    g.setParFile(str(p))
    g.configGeneratorFromFile()
    gr = g.grid()
    assert (gr["nm"], gr["ny"], gr["ymin"], gr["mmax"]) == (17, 9, -2.5, 20.0)
    # a missing file keeps the defaults (src/UpcGenerator.cpp:343-345)
    g2 = ug.UpcGenerator()
    g2.setParFile(str(tmp_path / "absent.in"))
    g2.configGeneratorFromFile()
    assert g2.grid()["nm"] == 1001 and g2.grid()["ny"] == 121


def test_bad_values_raise(ug):
    g = ug.UpcGenerator()
    with pytest.raises(ug.UpcgError):
        g.setParameterValue("BINS_M", "many")


@pytest.mark.parametrize("params,match", [
    ({"MMIN": 10, "MMAX": 5}, "mass range"),
    ({"PROC_ID": 51, "ALP_MASS": 0.01, "ALP_WIDTH": 0.01}, "mass range"),  # M - 4 Gamma < 0
    ({"YMIN": 3, "YMAX": -3}, "rapidity range"),
    ({"YMIN": float("nan")}, "rapidity range"),
    ({"ZMIN": 1, "ZMAX": -1}, "z range"),
    ({"SQRTS": 1.0}, "Lorentz factor"),
    ({"WS_A": 0}, "must be positive"),
    ({"NUCLEUS_A": 0}, "must be >= 1"),
    ({"BINS_M": 100000, "BINS_Y": 1000}, "at most"),
    ({"BINS_Y": 0}, "empty grid"),
    ({"BREAKUP_MODE": 5}, "BREAKUP_MODE"),
    ({"PROC_ID": 22}, "PROC_ID 22"),
])
def test_bad_configuration_refused_before_device_work(ug, params, match):
    """Values no table can be built from are refused by upcg_init on the host,
    before it looks for a device: the same error with or without a GPU."""
    g = ug.UpcGenerator(params)
    with pytest.raises(ug.UpcgError, match=match):
        g.init()


def test_compute_without_gpu_fails_loudly(ug):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    g = ug.UpcGenerator({"BINS_M": 3, "BINS_Y": 3})
    with pytest.raises(ug.UpcgError):
        g.init()


def test_event_output_config(ug, tmp_path):
    """NEVENTS, USE_ROOT_OUTPUT, USE_HEPMC_OUTPUT (src/UpcGenerator.cpp:185-187,
    284-289) from a parameter file; they leave the tables valid."""
    p = tmp_path / "parameters.in"
    p.write_text("NEVENTS 12345\nUSE_HEPMC_OUTPUT 1\nBINS_M 5\n")
    g = ug.UpcGenerator()
    # the reference's defaults: NEVENTS 1000, useROOTOut true, useHepMCOut
    # false (include/UpcGenerator.h:135-136)
    assert g.eventOutputConfig() == (1000, 1, 0)
    g.setParFile(str(p))
    g.configGeneratorFromFile()
    assert g.eventOutputConfig() == (12345, 1, 1)
    g.setParameterValue("USE_ROOT_OUTPUT", "0")
    assert g.eventOutputConfig() == (12345, 0, 1)
    assert g.candidateOffset() == 0
    with pytest.raises(ug.UpcgError):
        g.setParameterValue("NEVENTS", "lots")


def test_output_arrays_checked_on_the_host(ug):
    """The caller-owned out= arrays of generateEvents / lumiTable / nucCSYM
    are checked before any library call; page-locked memory needs a GPU."""
    import numpy as np
    import torch
    a = ug._out_array(None, (3, 4))
    assert a.shape == (3, 4) and a.dtype == np.float64 and not a.any()
    b = np.zeros((3, 4))
    assert ug._out_array(b, (3, 4)) is b
    for bad in (np.zeros((4, 3)), np.zeros((3, 4), dtype=np.float32), np.zeros((3, 8))[:, ::2]):
        with pytest.raises(ValueError):
            ug._out_array(bad, (3, 4))
    ro = np.zeros((3, 4))
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        ug._out_array(ro, (3, 4))
    g = ug.UpcGenerator({"BINS_M": 3, "BINS_Y": 3})
    with pytest.raises(ValueError):
        g.generateEvents(10, out=np.zeros(10, dtype=np.float32))
    with pytest.raises(ValueError):
        g.generateEvents(10, out=np.zeros(5, dtype=ug.EVENT_DTYPE))
    if not torch.cuda.is_available():
        with pytest.raises(ug.UpcgError):
            ug.pinned_array(16, ug.EVENT_DTYPE)


FACADE_PROGRAM = r"""
#include <cstdio>
#include "upcgen_gb300.hpp"
int main() {
  using namespace upcgen_gb300;
  UpcGenerator gen;
  gen.setParameterValue("PROC_ID", "13");
  gen.setParameterValue("BINS_M", "11");
  gen.setCollisionSystem(5360.f, 82, 208);
  int pdg = 0, charged = 0;
  check(upcg_particle_pdg(gen.handle(), &pdg, &charged));
  int thrown = 0;
  try {
    gen.setParameterValue("BINS_M", "not-a-number");
  } catch (const Error& e) {
    thrown = e.code() == UPCG_ERR_ARG;
  }
  int bad_format = 0;  // writeEvents: formats 0 (HepMC3) and 1 (columns) only
  try {
    gen.writeEvents("events.out", 1, 7);
  } catch (const Error& e) {
    bad_format = e.code() == UPCG_ERR_ARG;
  }
  // no file configured: the loop still needs the tables of init()
  gen.setParameterValue("USE_ROOT_OUTPUT", "0");
  int no_init = 0;
  try {
    gen.generateEvents();
  } catch (const Error& e) {
    no_init = e.code() == UPCG_ERR_STATE;
  }
  int not_vm = 0;  // calcNucCrossSectionY is the photonuclear path's
  try {
    UpcCrossSection cs(gen);
    double tot = 0;
    cs.calcNucCrossSectionY(5, nullptr, &tot);
  } catch (const Error& e) {
    not_vm = e.code() == UPCG_ERR_PROCESS;
  }
  std::printf("%d %d %d %d %d %d\n", pdg, charged, thrown, bad_format, not_vm, no_init);
  return 0;
}
"""


def test_cpp_facade_compiles_and_configures(ug, tmp_path):
    """include/upcgen_gb300.hpp: the reference's class names over the C ABI
    (configuration only -- no GPU here)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "facade.cpp"
    src.write_text(FACADE_PROGRAM)
    exe = tmp_path / "facade"
    lib = ug.library_path
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src),
                        lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["13", "1", "1", "1", "1", "1"]


def test_parameter_files_read_as_the_reference_reads_them(ug, tmp_path):
    """parameters.in files through configGeneratorFromFile against the
    reference's own reader and init, compiled from its sources
    (tests/golden/make_ref_config.py; fixture ref_config.json, and a live
    run when the sources are present): the grid after the process overrides
    (ALP mass window, dilepton MMIN clamp), NEVENTS and the output flags --
    with the reader's quirks: a key without a value takes the previous
    line's value, an indented '#' line reads as an unknown key, tokens after
    the value are ignored."""
    import json
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_ref_config as mk
    with open(os.path.join(os.path.dirname(__file__), "golden", "ref_config.json")) as f:
        fixture = json.load(f)
    assert set(fixture) == set(mk.FILES)
    from oracle import build as ob
    live = ob.build_ref_gen() is not None
    for name, text in mk.FILES.items():
        want = fixture[name]["reference"]
        assert fixture[name]["text"] == text
        if live:
            assert mk.run_fresh(name) == want, name
        p = tmp_path / f"{name}.in"
        p.write_text(text)
        g = ug.UpcGenerator()
        g.setParFile(str(p))
        g.configGeneratorFromFile()
        pdg, _ = g.particlePDG()  # applies the process overrides, as init does
        gr = g.grid()
        for k in ("mmin", "mmax", "ymin", "ymax", "zmin", "zmax", "nm", "ny", "nz"):
            assert gr[k] == want[k], (name, k, gr[k], want[k])
        assert g.eventOutputConfig() == (want["NEVENTS"], want["USE_ROOT_OUTPUT"],
                                         want["USE_HEPMC_OUTPUT"]), name
        assert pdg == want["PROC_ID"], name
