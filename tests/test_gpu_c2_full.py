"""Full-grid parity on the 1001 x 121 Pb-Pb table: Woods-Saxon form-factor
flux (FLUX_POINT 0), XnXn breakup (BREAKUP_MODE 2), m in [3.56, 50] GeV, y in
[-6, 6], every one of the 121,121 cells, the rapidity edges included.

The fixture tests/golden/c2_lumi.npz (tests/golden/make_c2_fixture.py) holds
the oracle's table twice:

* ``ref``: the reference's own quadrature -- fluxForm's QAGS at epsabs =
  epsrel = 1e-4 (src/UpcCrossSection.cpp:194-218), node layout and azimuth sum
  of calcTwoPhotonLumi (:221-271); the oracle equals the reference's compiled
  source on these (tests/test_oracle_pins.py);
* ``conv``: the same cells with the flux integral converged (QAGS at 1e-10).

The plain FP64 path reproduces ``ref`` to 1e-10 on all but a handful of
cells (8 of 121,121, 4 mirror pairs, up to 9.2e-10; median 6e-15): the
device's and the host's J1 and QAGS extrapolation differ in the last ulps,
and where the oscillating flux integral cancels those differences grow (the
reference's own GSL J1 is a third implementation); every cell is within 1e-9.  The fast form integrates the flux to convergence; it is
held to 1e-4 against ``conv`` on every cell above 1e-5 of the table's maximum
(99.99 % of its sum; measured 5.0e-5) and to stated bounds per magnitude band
below (the TeV photons at the rapidity edges, whose flux integral the
Q(w, b) table resolves less well: 1.9e-4 down to 1e-6 of the maximum, 1.2e-3
down to 1e-8, 3e-2 down to 1e-12, a factor 6.9 below), the cells beyond 1e-4
together 1.5e-7 of the table's sum.  Against ``ref`` it differs by more than
1e-4 on the cells where the reference's early QAGS stops do: ``ref`` itself
is more than 1e-4 away from ``conv`` on 142 of the 73,324 cells above 1e-5 of
the maximum (up to 0.118).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C2 = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "PROC_ID": 15, "LEP_A": 0, "FLUX_POINT": 0, "BREAKUP_MODE": 2,
      "MMIN": 3.56, "MMAX": 50, "BINS_M": 1001, "YMIN": -6, "YMAX": 6, "BINS_Y": 121,
      "ZMIN": -1, "ZMAX": 1, "BINS_Z": 100}
FAST_TOL = 1e-4
# the fast form on the cells below 1e-5 of the maximum (TeV photons): per band
# (lower edge as a fraction of the maximum, bound), from the measurement on
# this table with margin
FAST_BANDS = [(1e-6, 3e-4), (1e-8, 2e-3), (1e-12, 5e-2), (0.0, 10.0)]


@pytest.fixture(scope="module")
def fixture():
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "c2_lumi.npz"))
    return {k: d[k] for k in d.files}


def _table(ug, method):
    g = ug.UpcGenerator(C2)
    g.setLumiMethod(method)
    g.init()
    return g.lumiTable(), g.nucCSYM()[1]


def test_plain_full_grid_vs_reference_quadrature(ug, fixture):
    lumi, tot = _table(ug, "plain")
    ref = fixture["ref"]
    assert np.all(ref > 0)
    rel = np.abs(lumi / ref - 1)
    assert rel.max() <= 1e-9, (rel.max(), np.unravel_index(rel.argmax(), rel.shape))
    assert (rel > 1e-10).sum() <= 1e-4 * rel.size, int((rel > 1e-10).sum())
    assert np.median(rel) < 1e-13
    assert abs(tot / float(fixture["sigma_tot_ref"]) - 1) <= 1e-10


def test_fast_full_grid_vs_converged_quadrature(ug, fixture):
    lumi, tot = _table(ug, "fast")
    conv, ref = fixture["conv"], fixture["ref"]
    big = conv >= 1e-5 * conv.max()
    rel = np.abs(lumi / conv - 1)
    assert rel[big].max() <= FAST_TOL, (rel[big].max(), int(big.sum()))
    mx, hi = conv.max(), 1e-5
    for lo, bound in FAST_BANDS:
        band = (conv < hi * mx) & (conv >= lo * mx)
        assert rel[band].max() <= bound, (lo, hi, rel[band].max())
        hi = lo
    assert conv[~big].sum() / conv.sum() < 1e-5  # what the tiny cells weigh
    assert conv[rel > FAST_TOL].sum() / conv.sum() < 1e-6
    assert abs(tot / float(fixture["sigma_tot_conv"]) - 1) <= FAST_TOL
    assert abs(tot / float(fixture["sigma_tot_ref"]) - 1) <= FAST_TOL
    # against the reference's own quadrature: beyond 1e-4 only where the
    # reference is itself beyond 1e-4 of the converged integral, or by the
    # fast form's own error on top of it
    rel_ref = np.abs(lumi / ref - 1)
    noisy = np.abs(ref / conv - 1) > 0.5 * FAST_TOL
    assert np.all(rel_ref[big & ~noisy] <= 1.5 * FAST_TOL)
