"""The committed full-grid fixture tests/golden/c2_lumi.npz against the oracle
that made it (tests/golden/make_c2_fixture.py), on the CPU.

The GPU parity tests (tests/test_gpu_c2_full.py) read only the fixture; this
check keeps it tied to the oracle, and through tests/test_oracle_pins.py to
the reference's own src/UpcCrossSection.cpp: rows at the low, middle and top
of the mass range, every rapidity (the +-6 edges included), recomputed
bit-exact for both tables (the reference's QAGS at 1e-4 and the converged
flux integral), and the stored sigma_tot values equal to the oracle's fold
(calcNucCrossSectionYM, src/UpcCrossSection.cpp:594-698) of the stored
tables.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_c2_fixture import C2, CONV_EPS  # noqa: E402


@pytest.fixture(scope="module")
def fixture():
    d = np.load(os.path.join(HERE, "golden", "c2_lumi.npz"))
    return {k: d[k] for k in d.files}


@pytest.mark.parametrize("key,rows", [("ref", (0, 500, 1000)), ("conv", (0, 1000))])
def test_fixture_rows_are_the_oracle(oracle_mod, fixture, key, rows):
    params = dict(C2) if key == "ref" else dict(C2, ORACLE_FLUX_EPS=CONV_EPS)
    assert float(fixture["conv_eps"]) == CONV_EPS
    o = oracle_mod.Oracle(params, threads=os.cpu_count() or 1)
    o.init_tables()
    assert fixture[key].shape == (1001, 121)
    for im in rows:
        got = o.lumi_table(im, im + 1)
        assert np.array_equal(got, fixture[key][im:im + 1]), (key, im)


def test_fixture_sigma_tot_is_the_fold(oracle_mod, fixture):
    o = oracle_mod.Oracle(C2, threads=1)
    o.init_tables()
    for key in ("ref", "conv"):
        _, tot, _ = o.nuc_cs_ym(fixture[key])
        assert tot == float(fixture["sigma_tot_" + key]), (key, tot)
    # the two quadratures differ by far less than the fast form's 1e-4 budget
    # on sigma_tot, although single cells differ by up to 0.118
    assert abs(float(fixture["sigma_tot_ref"]) / float(fixture["sigma_tot_conv"]) - 1) < 1e-5
