"""Photonuclear path on the GPU against the oracle: calcPhotonFlux,
UpcPhotoNuclearVM::calcCrossSectionY (impulse approximation) and
calcNucCrossSectionY at relative 1e-10, and vector-meson events (y, meson pT,
decay angle, emitter choice) chi2-tested against the oracle's events, which
draw the pomeron pT and the decay angle by the reference's rejection loops."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JPSI = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
        "PROC_ID": 443, "DECAY_PDG": 13, "FLUX_POINT": 0, "BREAKUP_MODE": 1,
        "YMIN": -6, "YMAX": 6, "BINS_Y": 121, "SEED": 3}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def _pair(ug, oracle_mod, p):
    g = ug.UpcGenerator(p)
    g.init()
    o = oracle_mod.Oracle(p, threads=os.cpu_count())
    o.init_tables()
    return g, o


@pytest.mark.parametrize("extra", [{}, {"FLUX_POINT": 1}, {"BREAKUP_MODE": 2},
                                   {"PROC_ID": 553, "DECAY_PDG": 11, "BREAKUP_MODE": 4},
                                   {"PROC_ID": 100443, "DECAY_PDG": 2212, "NUCLEUS_Z": 79,
                                    "NUCLEUS_A": 197, "WS_R": 6.38, "WS_A": 0.535, "SQRTS": 200}],
                         ids=["jpsi-ff", "jpsi-point", "jpsi-xnxn", "upsilon-0n0n", "psi2s-au"])
def test_flux_sigma_and_nuclear_cs(ug, oracle_mod, extra):
    p = dict(JPSI, **extra)
    g, o = _pair(ug, oracle_mod, p)
    mV = g.grid()["mmin"] + 1e-6
    y = np.linspace(-6, 6, 37)
    # Where the flux has fallen below 1e-12 of its peak (photon energies near
    # the gamma hc / b cut-off) the form-factor integral cancels to roundoff
    # and both implementations return noise: compare above that.
    f, fo = g.calcPhotonFlux(mV, y), np.array([o.photon_flux(mV, v) for v in y])
    keep = fo > 1e-12 * fo.max()
    assert keep.sum() >= 20 and rel(f[keep], fo[keep]) < 1e-10
    assert rel(g.vmCrossSectionY(y), [o.vm_cs_y(v) for v in y]) < 1e-10
    cs, ratio, tot = g.nucCSY()
    rcs, rratio, rtot = o.nuc_cs_y()
    # the same noise in bins whose dsigma/dy comes from such fluxes, and in the
    # ratio's small side
    big = rcs > 1e-12 * rcs.max()
    both = (rratio > 1e-12) & (rratio < 1e12)
    assert rel(cs[big], rcs[big]) < 1e-10 and rel(ratio[both], rratio[both]) < 1e-10
    assert abs(tot / rtot - 1) < 1e-10
    assert g.totNuclX() == tot
    assert g.qagsStats()["failures"] == 0


def _chi2_two_sample(a, b, bins):
    from scipy import stats
    ha, _ = np.histogram(a, bins)
    hb, _ = np.histogram(b, bins)
    na, nb = ha.sum(), hb.sum()
    keep = (ha + hb) > 0
    ha, hb = ha[keep].astype(float), hb[keep].astype(float)
    chi2 = np.sum((ha * np.sqrt(nb / na) - hb * np.sqrt(na / nb)) ** 2 / (ha + hb))
    return stats.chi2.sf(chi2, keep.sum() - 1)


def _decay_cos(p0, p1):
    """cos of the first daughter's angle to the meson direction, in the meson frame."""
    P = p0 + p1
    M = np.sqrt(np.maximum(P[:, 3] ** 2 - (P[:, :3] ** 2).sum(1), 0))
    b = P[:, :3] / P[:, 3:4]
    b2 = (b ** 2).sum(1)
    gam = P[:, 3] / M
    bp = (b * p0[:, :3]).sum(1)
    g2 = np.where(b2 > 0, (gam - 1) / np.where(b2 > 0, b2, 1), 0)
    v = p0[:, :3] + (g2 * bp - gam * p0[:, 3])[:, None] * b  # boost by -beta
    u = P[:, :3] / np.linalg.norm(P[:, :3], axis=1, keepdims=True)
    return (v * u).sum(1) / np.linalg.norm(v, axis=1)


@pytest.mark.parametrize("extra", [{}, {"DECAY_PDG": 2212, "DO_ETA_CUT": 1, "ETA_MIN": -2.5,
                                        "ETA_MAX": 2.5, "DO_PT_CUT": 1, "PT_MIN": 0.02}],
                         ids=["jpsi-mumu", "jpsi-ppbar-cuts"])
def test_vm_events(ug, oracle_mod, extra):
    p = dict(JPSI, BINS_Y=61, **extra)
    g, o = _pair(ug, oracle_mod, p)
    cs, ratio, tot = o.nuc_cs_y()
    # the oracle draws the pomeron pT as the reference does, by rejection with
    # ~2e4 form-factor evaluations per event: a few thousand events
    n_o = 4000
    rec, rej_o, _ = o.generate(cs.reshape(-1, 1), np.zeros(1), n_o, 11, ratio=ratio)
    n = 400000
    ev, rej_g = g.generateEvents(n)
    p0o, p1o = rec[:, 4:8], rec[:, 8:12]
    p0g, p1g = ev["p0"].astype(np.float64), ev["p1"].astype(np.float64)
    Po, Pg = p0o + p1o, p0g + p1g
    checks = {
        "y": (ev["y"], rec[:, 1], np.linspace(-6, 6, 25)),
        "pt": (np.hypot(Pg[:, 0], Pg[:, 1]), np.hypot(Po[:, 0], Po[:, 1]), np.linspace(0, 0.3, 31)),
        "cos": (_decay_cos(p0g, p1g), _decay_cos(p0o, p1o), np.linspace(-1, 1, 21)),
        "sign": (ev["sign"], rec[:, 3], np.array([-2, 0, 2])),
        "daughter_pt": (np.hypot(p0g[:, 0], p0g[:, 1]), np.hypot(p0o[:, 0], p0o[:, 1]),
                        np.linspace(0, 2.5, 26)),
    }
    for name, (a, b, bins) in checks.items():
        pv = _chi2_two_sample(a, b, bins)
        assert pv > 1e-4, f"{name}: chi2 p-value {pv:.2e}"
    # the pair's invariant mass is the meson's (float32 momenta: checked where
    # E < 31 GeV, so that E^2 - p^2 keeps its digits)
    M = np.sqrt(np.maximum(Pg[:, 3] ** 2 - (Pg[:, :3] ** 2).sum(1), 0))
    central = np.abs(ev["y"]) < 3
    assert central.sum() > n // 4 and np.allclose(M[central], 3.0969, rtol=1e-3)
    if extra:
        fa, fb = n / (n + rej_g), n_o / (n_o + rej_o)
        sig = np.sqrt(fa * (1 - fa) / (n + rej_g) + fb * (1 - fb) / (n_o + rej_o))
        assert abs(fa - fb) < 5 * sig
        pt = np.hypot(Pg[:, 0], Pg[:, 1])
        assert pt.min() >= 0.02 * (1 - 1e-5)
    assert g.particlesPerEvent() == 3 and g.decayPDG() == p["DECAY_PDG"]


def test_vm_refusals(ug):
    g = ug.UpcGenerator(dict(JPSI, SHADOWING=1))
    with pytest.raises(ug.UpcgError, match="SHADOWING"):
        g.init()
    g = ug.UpcGenerator(dict(JPSI, BINS_Y=11))
    g.init()
    with pytest.raises(ug.UpcgError, match="two-photon luminosity"):
        g.lumiTable()
