"""Pins of the CPU oracle (no GPU).

ROOT and GSL are not installed, so the reference cannot be built with its own
build system.  The oracle is pinned
(1) against the reference's own elementary cross sections, compiled from its
sources (golden ref_elem.json, bit for bit);
(2) against the reference's own UpcCrossSection -- src/UpcCrossSection.cpp
compiled where it lies against the GSL / ROOT stand-ins of oracle/refshim/,
whose spline, QAGS and Bessel calls are the oracle's own primitives -- on
rho0, G_AA, the form factor, both fluxes, the breakup probability and its
spline, the luminosity cells (unpolarized and polarized, grid edges included)
and the photonuclear flux, bit for bit (golden ref_cs.json, and the live
build when the reference sources are present);
(3) primitive by primitive against scipy; and
(4) against the independent numpy/scipy restatement in
tests/golden/make_golden.py (golden numpy_restatement.json).
"""
import json
import os

import numpy as np
import pytest
from scipy import integrate, interpolate, special

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_elementary_cs_bit_exact_vs_reference(oracle_mod):
    g = load("ref_elem.json")
    for e in g["dilep"]:
        o = oracle_mod.Oracle({"PROC_ID": e["pdg"], "LEP_A": e["alep"]})
        o.init_tables()
        for flag in (0, 1, 2):
            assert o.cs_m(e["m"], flag) == e["cs_m"][flag]
            for z, v in zip(e["z"], e["cs_zm"][flag]):
                got = o.cs_zm(z, e["m"], flag)
                assert got == v or (np.isnan(got) and np.isnan(v)), (e["pdg"], flag, z, got, v)
    for e in g["alp"]:
        o = oracle_mod.Oracle({"PROC_ID": 51, "ALP_MASS": e["mass"], "ALP_WIDTH": e["width"]})
        o.init_tables()
        assert o.cs_m(e["m"], 0) == e["cs_m"]


def test_live_reference_elementary(oracle_mod):
    L = oracle_mod.ref_lib()
    if L is None:
        pytest.skip("reference sources not present on this machine")
    o = oracle_mod.Oracle({"PROC_ID": 15})
    o.init_tables()
    for m in np.geomspace(3.56, 50, 23):
        assert o.cs_m(m, 0) == L.uref_dilep_cs_m(15, 0.0, m, 0)
        for z in np.linspace(-0.99, 0.99, 9):
            assert o.cs_zm(z, m, 0) == L.uref_dilep_cs_zm(15, 0.0, z, m, 0)


def _check_ref_cs(oracle_mod, e, ref=None):
    """The oracle against one configuration of ref_cs.json (bit for bit);
    `ref`: the live reference build, checked at the same points as well."""
    p = e["params"]
    o = oracle_mod.Oracle(p, threads=4)
    o.init_tables()
    mode = p["BREAKUP_MODE"]
    got = {"rho0": o.rho0()}
    assert o.rho0() == e["rho0"]
    for b, v in e["gaa_spline"]:
        assert o.gaa(b) == v, ("gaa", b)
    for q2, v in e["form_factor"]:
        assert o.form_factor(q2) == v, ("ff", q2)
    for b, k, v in e["flux_point"]:
        assert o.flux_point(b, k) == v, ("flux_point", b, k)
    for b, k, v in e["flux_form"]:
        assert o.flux_form(b, k) == v, ("flux_form", b, k)
    for b, v in e["breakup_prob"]:
        assert o.breakup_prob(b, mode) == v, ("breakup", b)
    for b, v in e.get("breakup_spline", []):
        assert o.breakup_spline(b) == v, ("breakup spline", b)
    for im, iy, m, y, v in e.get("lumi", []):
        assert o.two_photon_lumi(m, y) == v, ("lumi", im, iy)
    for im, iy, m, y, vs, vp in e.get("lumi_pol", []):
        assert o.two_photon_lumi_pol(m, y) == (vs, vp), ("lumi pol", im, iy)
    for m, y, v in e["photon_flux"]:
        assert o.photon_flux(m, y) == v, ("photon flux", m, y)
    if ref is not None:
        assert ref.rho0() == got["rho0"]
        for im, iy, m, y, v in e.get("lumi", []):
            assert ref.two_photon_lumi(m, y) == v
        for im, iy, m, y, vs, vp in e.get("lumi_pol", []):
            assert ref.two_photon_lumi_pol(m, y) == (vs, vp)


@pytest.mark.parametrize("name", ["pb_point_mode1", "pb_point_mode2", "pb_point_mode3",
                                  "pb_point_mode4", "pb_form_mode2", "pb_form_mode2_pol",
                                  "au200_form_mode4", "o16_form_mode3_alp"])
def test_oracle_bit_exact_vs_reference_cross_section(oracle_mod, name):
    """The oracle equals the reference's own UpcCrossSection (compiled from
    src/UpcCrossSection.cpp; tests/golden/make_ref_cs.py) bit for bit:
    calcWSRho, prepareGAA, calcFormFac, fluxPoint, fluxForm (QAGS at 1e-4),
    calcBreakupProb / prepareBreakupProb, calcTwoPhotonLumi(Pol) on cells at
    the grid's edges, calcPhotonFlux."""
    _check_ref_cs(oracle_mod, load("ref_cs.json")["configs"][name])


def _live_check(name):
    from oracle import oracle
    e = load("ref_cs.json")["configs"][name]
    _check_ref_cs(oracle, e, oracle.RefCrossSection(e["params"]))
    return True


@pytest.mark.parametrize("name", ["pb_form_mode2", "au200_form_mode4"])
def test_live_reference_cross_section(oracle_mod, name):
    """The same against a live build of the reference's sources (skipped where
    they are absent): the fixture is what the reference's code computes today.
    Each configuration runs in a fresh process, as the reference needs
    (calcBreakupProb builds its tables once per process)."""
    if oracle_mod.ref_cs_lib() is None:
        pytest.skip("reference sources not present on this machine")
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(1, mp_context=mp.get_context("spawn")) as ex:
        assert ex.submit(_live_check, name).result()


def test_bessel_k_vs_scipy(oracle_mod):
    x = np.concatenate([np.geomspace(1e-9, 2, 300), np.linspace(2, 30, 300), np.linspace(30, 700, 100)])
    for xi in x:
        k0, k1 = oracle_mod.bessel_k01(float(xi))
        assert k0 == pytest.approx(special.k0(xi), rel=5e-15, abs=0)
        assert k1 == pytest.approx(special.k1(xi), rel=5e-15, abs=0)


def test_abramowitz_stegun_k1(oracle_mod):
    # A&S 9.8.7/9.8.8 quote |error| < 8e-9 (x K1 e^x scale); relative ~2e-7
    for xi in np.geomspace(1e-6, 50, 400):
        assert oracle_mod.bessel_k1_as(float(xi)) == pytest.approx(special.k1(xi), rel=3e-7)


def test_gauss_kronrod_exactness():
    from numpy.polynomial import legendre
    xg = np.array([0.995657163025808080735527280689003, 0.973906528517171720077964012084452,
                   0.930157491355708226001207180059508, 0.865063366688984510732096688423493,
                   0.780817726586416897063717578345042, 0.679409568299024406234327365114874,
                   0.562757134668604683339000099272694, 0.433395394129247190799265943165784,
                   0.294392862701460198131126603103866, 0.148874338981631210884826001129720, 0.0])
    wk = np.array([0.011694638867371874278064396062192, 0.032558162307964727478818972459390,
                   0.054755896574351996031381300244580, 0.075039674810919952767043140916190,
                   0.093125454583697605535065465083366, 0.109387158802297641899210590325805,
                   0.123491976262065851077208980430855, 0.134709217311473325928054001771707,
                   0.142775938577060080797094273138717, 0.147739104901338491374841515972068,
                   0.149445554002916905664936468389821])
    wg = np.array([0.066671344308688137593568809893332, 0.149451349150580593145776339657697,
                   0.219086362515982043995534934228163, 0.269266719309996355091226921569469,
                   0.295524224714752870173892994651338])
    xs = np.concatenate([-xg[:10], xg[::-1]])
    ws = np.concatenate([wk[:10], wk[::-1]])
    for p in range(0, 32):
        exact = 0.0 if p % 2 else 2.0 / (p + 1)
        assert np.dot(ws, xs ** p) == pytest.approx(exact, abs=1e-14)
    gx, gw = legendre.leggauss(10)
    assert np.allclose(np.sort(np.abs(gx))[::2], np.sort(xg[1:10:2]), atol=1e-15)
    assert np.allclose(np.sort(gw)[::2], np.sort(wg), atol=1e-15)


@pytest.mark.parametrize("fid,p0,p1,a,b", [
    (0, 2.5, 0, 0.0, 1.0), (1, 7.0, 0.3, 0.0, 10.0), (2, -0.5, 0, 0.0, 1.0),
    (3, 30.0, 0.01, 0.0, 10.0), (3, 400.0, 1e-4, 0.0, 10.0)])
def test_qags_vs_quadpack(oracle_mod, fid, p0, p1, a, b):
    f = {0: lambda x: x ** p0, 1: lambda x: np.cos(p0 * x) * np.exp(-p1 * x),
         2: lambda x: x ** p0 * np.log(x), 3: lambda x: x * x / (x * x + p1) * special.j1(p0 * x)}[fid]
    r, e, ne, ni, st = oracle_mod.qags_test(fid, p0, p1, a, b, 1e-4, 1e-4)
    q = integrate.quad(f, a, b, epsabs=1e-4, epsrel=1e-4, limit=1000, full_output=1)
    assert st == 0
    # same algorithm: same number of evaluations; results agree to rounding
    # (extrapolated results to the extrapolation's own accuracy)
    assert ne == q[2]["neval"]
    assert r == pytest.approx(q[0], rel=1e-9, abs=1e-12)


def test_spline_vs_scipy(oracle_mod):
    rng = np.random.default_rng(3)
    x = np.cumsum(rng.uniform(0.1, 1.0, 300))
    y = np.sin(x) * np.exp(-0.01 * x)
    xe = np.sort(rng.uniform(x[0], x[-1], 1000))
    ref = interpolate.CubicSpline(x, y, bc_type="natural")(xe)
    assert np.allclose(oracle_mod.spline_natural(x, y, xe), ref, rtol=0, atol=1e-13)


def test_simpson_weights(oracle_mod):
    v = np.arange(10.0) ** 2
    h = 0.5
    expected = (v[0] + v[-1] + 4 * v[1:-1:2].sum() + 2 * v[2:-1:2].sum()) * h / 3
    assert oracle_mod.simpson(v, h) == expected


def test_sampler_bin_truncation(oracle_mod):
    # include/UpcSampler.h:124-134: int(n*(x-x0)) / (x1-x0), truncated again
    for x in np.random.default_rng(5).uniform(3.56, 50.0, 2000):
        expected = int(int(1001 * (x - 3.56)) / (50.0 - 3.56))
        assert oracle_mod.sampler_bin(1001, 3.56, 50.0, float(x)) == expected
    # differs from the plain bin index for some masses (the reference's quirk)
    xs = np.linspace(3.56, 49.99, 20011)
    plain = np.floor((xs - 3.56) / (50 - 3.56) * 1001).astype(int)
    quirk = np.array([oracle_mod.sampler_bin(1001, 3.56, 50.0, float(x)) for x in xs])
    assert np.any(plain != quirk) and np.all(np.abs(plain - quirk) <= 1)


class TestNumpyRestatement:
    g = load("numpy_restatement.json")

    @pytest.fixture(scope="class")
    def o(self, oracle_mod):
        o = oracle_mod.Oracle({"PROC_ID": 15, "BREAKUP_MODE": 2, "FLUX_POINT": 0})
        o.init_tables()
        return o

    def test_rho0_gaa(self, o):
        assert o.rho0() == pytest.approx(self.g["rho0"], rel=1e-14)
        for b, v in zip(self.g["gaa"]["b"], self.g["gaa"]["v"]):
            # G_AA spans 300 decades; below ~1e-20 the spline is rounding-level
            assert o.gaa(b) == pytest.approx(v, rel=1e-11, abs=1e-14)

    def test_form_factor(self, o):
        ff = self.g["form_factor"]
        for q2, v, s in zip(ff["q2"], ff["v"], ff["spline"]):
            assert o.form_factor(q2) == pytest.approx(v, rel=1e-9)
            assert o.form_factor_spline(q2) == pytest.approx(s, rel=1e-9)

    def test_breakup(self, o):
        br = self.g["breakup"]
        for mode, vals in br["modes"].items():
            for b, v in zip(br["b"], vals):
                assert o.breakup_prob(b, int(mode)) == pytest.approx(v, rel=1e-11, abs=1e-300)
        sp = self.g["breakup_spline_xnxn"]
        for b, v in zip(sp["b"], sp["v"]):
            assert o.breakup_spline(b) == pytest.approx(v, rel=1e-11, abs=1e-300)

    def test_flux_form(self, o):
        for e in self.g["flux_form"]:
            assert o.flux_form(e["b"], e["k"]) == pytest.approx(e["v"], rel=1e-9)

    def test_lumi_cells(self, oracle_mod):
        for c in self.g["lumi_cells"]:
            o = oracle_mod.Oracle({"PROC_ID": 13, "FLUX_POINT": c["flux_point"], "BREAKUP_MODE": c["mode"]})
            o.init_tables()
            assert o.two_photon_lumi(c["M"], c["Y"]) == pytest.approx(c["L"], rel=1e-10)


def test_breakup_mode_identity(oracle_mod):
    # modes 2 + 3 + 4 sum to one: (1-e)^2 + e^2 + 2e(1-e) = 1
    o = oracle_mod.Oracle({"PROC_ID": 13})
    o.init_tables()
    for b in np.geomspace(1e-3, 900, 60):
        s = sum(o.breakup_prob(b, m) for m in (2, 3, 4))
        assert s == pytest.approx(1.0, abs=1e-15)


def test_gaa_limits(oracle_mod):
    o = oracle_mod.Oracle({"PROC_ID": 13})
    o.init_tables()
    assert o.gaa(0.0) < 1e-100          # central collisions never survive
    assert o.gaa(19.99) == pytest.approx(1.0, abs=2e-4)
    w = np.array([0.2955242247147529, 0.2692667193099963, 0.2190863625159820,
                  0.1494513491505806, 0.0666713443086881])
    assert w.sum() == pytest.approx(0.9999999999999999, abs=2e-16)


def test_reference_flux_quadrature_noise(oracle_mod):
    """The reference's form-factor flux QAGS (epsabs = epsrel = 1e-4,
    src/UpcCrossSection.cpp:209) stops early at some nodes: at b = 4.5545 fm,
    k = 10.75 GeV it returns a flux 5 % above the converged integral.  With
    ORACLE_FLUX_EPS = 1e-10 the oracle's flux agrees with an independent
    adaptive quadrature (scipy) to 1e-9."""
    p = {"PROC_ID": 15, "FLUX_POINT": 0, "BREAKUP_MODE": 2}
    o = oracle_mod.Oracle(p)
    o.init_tables()
    oc = oracle_mod.Oracle(dict(p, ORACLE_FLUX_EPS=1e-10))
    oc.init_tables()
    b, k = 4.5545, 10.75
    g, hc, A = o.gamma(), 0.1973269718, 208
    q2c = 2 - (2 - 1e-9) / 1e6

    def integrand(q):
        t = q * q + (k / g) ** 2
        return q * q * o.form_factor_spline(t if t < 2 else q2c) / t * special.j1(b * q / hc)

    v, _ = integrate.quad(integrand, 0, 10, epsabs=1e-13, epsrel=1e-12, limit=5000)
    fconv = oc.flux_form(b, k)
    fref = o.flux_form(b, k)
    scale = fconv / (v / A) ** 2 * k  # the flux's constant factor
    assert scale == pytest.approx(82 ** 2 / 137.035999074 / np.pi ** 2 / hc ** 2, rel=1e-9)
    assert fref / fconv - 1 == pytest.approx(0.0527, abs=2e-3)


VM = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "PROC_ID": 443, "DECAY_PDG": 13, "FLUX_POINT": 0, "BREAKUP_MODE": 2, "BINS_Y": 9}


def test_vm_cross_section_restatement(oracle_mod):
    """UpcPhotoNuclearVM::calcCrossSectionY (src/UpcPhotoNuclearVM.cpp:42-53,
    340-381, impulse approximation) recomputed with scipy's quad: dsdt closed
    form times the integral of calcFormFac^2 over [tmin, tmin + 1]."""
    o = oracle_mod.Oracle(VM)
    o.init_tables()
    mV, mp, mn = 3.0969, 0.9382720813, 0.939565346
    mnucl = (82 * mp + 126 * mn) / 208
    for y in (-4.0, -1.5, 0.0, 2.0, 5.0):
        w = mV / 2 * np.exp(y)
        W2 = 4 * w * 2510.0
        wmin = mp + mV
        cs = 342.0 * (1 - wmin ** 2 / W2) ** 1.5 * (W2 * 1e-4) ** 0.4 if np.sqrt(W2) > wmin else 0.0
        tmin = (mV ** 2 / W2) ** 2 * mnucl ** 2
        edges = np.linspace(np.sqrt(tmin), np.sqrt(tmin + 1), 41)
        phi = sum(integrate.quad(lambda q: o.form_factor(q * q) ** 2 * 2 * q, a, b,
                                 epsabs=0, epsrel=1e-13, limit=200)[0]
                  for a, b in zip(edges[:-1], edges[1:]))
        assert o.vm_cs_y(y) == pytest.approx(cs * phi * 1e-6, rel=1e-11)


def test_photon_flux_restatement(oracle_mod):
    """calcPhotonFlux (src/UpcCrossSection.cpp:700-722) as a Python loop over
    the oracle's fluxForm, G_AA and breakup splines."""
    o = oracle_mod.Oracle(VM)
    o.init_tables()
    R, g1, hc = 6.68, 5020 / (2 * 0.9382720813), 0.1973269718
    for m, y in ((3.0969, -3.0), (3.0969, 0.5), (9.3987, 2.5)):
        k = m / 2 * np.exp(y)
        bmin, bmax = 0.05 * R, max(5 * g1 * hc / k, 5 * R)
        ldb = (np.log(bmax) - np.log(bmin)) / 120
        s = 0.0
        for i in range(120):
            bl, bh = bmin * np.exp(i * ldb), bmin * np.exp((i + 1) * ldb)
            b = (bh + bl) / 2
            bu = o.breakup_spline(min(b, 20.0))
            ga = o.gaa(b) if b < 20 else 1.0
            s += bu * ga * o.flux_form(b, k) * b * (bh - bl)
        assert o.photon_flux(m, y) == pytest.approx(2 * np.pi * k * s, rel=1e-13)
