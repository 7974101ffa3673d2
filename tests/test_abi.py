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


def test_compute_without_gpu_fails_loudly(ug):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    g = ug.UpcGenerator({"BINS_M": 3, "BINS_Y": 3})
    with pytest.raises(ug.UpcgError):
        g.init()
