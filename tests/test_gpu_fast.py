"""Fast form (tensor-core contraction) against the FP64 oracle.

Budget: 1e-4 relative per luminosity cell and on sigma_tot.  The fast form
keeps the reference's per-cell impact-parameter nodes; its error comes from
the survival kernel's interpolation on the fixed radial grid, the flux
tables, and the BF16 hi/lo split with FP32 accumulation.

With the form-factor flux the reference integrates each node's flux by QAGS
at epsabs = epsrel = 1e-4 (src/UpcCrossSection.cpp:209).  That quadrature
stops early on the oscillating Bessel integrand at some nodes (at b = 4.55
fm, k = 10.75 GeV it returns a flux 5 % above the converged integral), so the
reference's own cells carry errors of up to a few 1e-4 in the bulk and
factors at the rapidity edges, where the photon energy reaches TeV.  The
fast form integrates to convergence; its cells are checked against the
oracle run with a converged flux quadrature (ORACLE_FLUX_EPS = 1e-10), and
its sigma_tot against the reference's.  On the 1001 x 121 Pb-Pb form-factor
table the fast form stays within 1.7e-5 of the converged quadrature on every
cell above 1e-4 of the maximum and within 5.1e-5 above 1e-5, where the
reference's own cells are off by up to 6e-2 and 1.2e-1.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FAST_TOL = 1e-4

C1 = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "PROC_ID": 13, "LEP_A": 0, "FLUX_POINT": 1, "BREAKUP_MODE": 1,
      "MMIN": 3.56, "MMAX": 50, "BINS_M": 201, "YMIN": -6, "YMAX": 6, "BINS_Y": 61,
      "ZMIN": -1, "ZMAX": 1, "BINS_Z": 100, "SEED": 1}


@pytest.mark.parametrize("ncells,P", [(256, 256), (1000, 1024)])
def test_contraction_vs_fp64(ug, ncells, P):
    err, ms = ug.selftest_contract(ncells, P, seed=3)
    assert err >= 0, f"contraction kernel error word {-err}"
    # hi*hi + hi*lo + lo*hi of the same bf16 pairs, FP32 accumulation
    assert err < 2e-5, err


def _fast_vs_oracle(ug, oracle_mod, params):
    g = ug.UpcGenerator(params)
    g.setLumiMethod("fast")
    g.init()
    lumi = g.lumiTable()
    o = oracle_mod.Oracle(params, threads=os.cpu_count())
    o.init_tables()
    ref = o.lumi_table()
    if params.get("FLUX_POINT", 1):
        conv = ref  # closed-form flux: no quadrature noise in the reference
    else:
        oc = oracle_mod.Oracle(dict(params, ORACLE_FLUX_EPS=1e-10), threads=os.cpu_count())
        oc.init_tables()
        conv = oc.lumi_table()
    rel = np.abs(lumi - conv) / np.abs(conv)
    if not params.get("FLUX_POINT", 1):
        # At photon energies of TeV the reference's flux integral is dominated
        # by its cut at q = 10 GeV (J1 ripples of period 0.12 fm in b), which
        # the Q(w, b) table does not resolve; those cells lie below 1e-5 of
        # the table's maximum (together < 1e-5 of its sum) and are left out.
        rel = rel[np.abs(conv) >= 1e-5 * np.abs(conv).max()]
    _, tot = g.nucCSYM()
    _, rtot, _ = o.nuc_cs_ym(ref)
    return rel, abs(tot / rtot - 1), g


def test_fast_config1_full_grid(ug, oracle_mod):
    rel, rtot, g = _fast_vs_oracle(ug, oracle_mod, C1)
    assert rel.max() < FAST_TOL, (rel.max(), np.unravel_index(rel.argmax(), rel.shape))
    assert rtot < FAST_TOL
    t = g.timings()
    assert t["contract_ms"] > 0
    # the contraction's work: the rows computed, and per row the multiply-adds
    # over the tiles where the survival kernel minus its constant can be
    # nonzero -- whole tiles of 64 x 128 or 64 x 256, fewer than the dense
    # 1024^2 (the tiles below the first node stencil and those where every
    # azimuth reaches b >= 20 fm are skipped)
    rows, macs = g.contractWork()
    assert rows == g.contractRows() > 0
    assert 0 < macs < 1024 * 1024 and macs % (64 * 128) == 0, macs
    # one cell of each mirror pair y_j = -y_i (i + j = 61 on this grid; left
    # edges equal and opposite to 8 ulps) is computed and the other copied:
    # L(m, -y) = L(m, y).  Pairs whose edges miss the 8-ulp match are both
    # computed and agree to the fast form's rounding.
    lumi = g.lumiTable()
    a, b = lumi[:, 1:], lumi[:, 1:][:, ::-1]
    assert np.allclose(a, b, rtol=2e-5, atol=0)
    assert np.mean(np.all(a == b, axis=0)) > 0.8


@pytest.mark.parametrize("mode", [2, 3, 4])
def test_fast_breakup_modes(ug, oracle_mod, mode):
    rel, rtot, _ = _fast_vs_oracle(ug, oracle_mod, dict(C1, BREAKUP_MODE=mode, BINS_M=41, BINS_Y=25))
    assert rel.max() < FAST_TOL and rtot < FAST_TOL


def test_fast_form_factor_flux(ug, oracle_mod):
    p = dict(C1, PROC_ID=15, FLUX_POINT=0, BREAKUP_MODE=2, BINS_M=21, BINS_Y=13)
    rel, rtot, _ = _fast_vs_oracle(ug, oracle_mod, p)
    assert rel.max() < FAST_TOL and rtot < FAST_TOL


@pytest.mark.parametrize("flux_point", [1, 0])
def test_fast_polarized(ug, oracle_mod, flux_point):
    """USE_POLARIZED_CS in the fast form: the scalar and pseudoscalar survival
    kernels (b^2 = b1^2 + b2^2 - 2 b1 b2 cos phi, weights cos^2 / sin^2 phi;
    src/UpcCrossSection.cpp:274-335) in two contractions of the same operands;
    both tables within 1e-4 of the (converged) oracle."""
    p = dict(C1, PROC_ID=13, BREAKUP_MODE=2, USE_POLARIZED_CS=1, FLUX_POINT=flux_point,
             BINS_M=21, BINS_Y=25)
    g = ug.UpcGenerator(p)
    g.setLumiMethod("fast")
    g.init()
    s, ps = g.lumiTable(polarized=True)
    o = oracle_mod.Oracle(dict(p, ORACLE_FLUX_EPS=1e-10) if not flux_point else p,
                          threads=os.cpu_count())
    o.init_tables()
    rs, rp = o.lumi_table(polarized=True)
    for a, b in ((s, rs), (ps, rp)):
        big = np.abs(b) >= 1e-5 * np.abs(b).max()
        assert (np.abs(a - b)[big] / np.abs(b[big])).max() < FAST_TOL
    # sigma and the scalar / pseudoscalar ratio of the fold
    _, tot = g.nucCSYM()
    _, rtot, _ = o.nuc_cs_ym(rs, rp)
    assert abs(tot / rtot - 1) < FAST_TOL


def test_fast_light_nucleus(ug, oracle_mod):
    p = dict(C1, PROC_ID=51, ALP_MASS=1, ALP_WIDTH=0.01, NUCLEUS_Z=8, NUCLEUS_A=16,
             WS_R=2.608, WS_A=0.513, SQRTS=5360, BREAKUP_MODE=3, BINS_M=21, BINS_Y=25)
    rel, rtot, _ = _fast_vs_oracle(ug, oracle_mod, p)
    assert rel.max() < FAST_TOL and rtot < FAST_TOL


@pytest.mark.parametrize("mode", [2, 3, 4])
def test_fast_breakup_table_fp32(ug, mode):
    """The fast form's breakup table comes from FP32 trapezoid sums: within
    1e-5 of the FP64 table (the plain path's), absolutely and relative to
    values above 1e-3."""
    b = np.linspace(1e-6, 20.0, 4001)
    vals = {}
    for meth in ("plain", "fast"):
        g = ug.UpcGenerator(dict(C1, BREAKUP_MODE=mode, BINS_M=3, BINS_Y=3))
        g.setLumiMethod(meth)
        g.init()
        vals[meth] = g.nucProcessCS.spline("breakup", b)
    d = np.abs(vals["fast"] - vals["plain"])
    assert d.max() < 1e-5
    big = np.abs(vals["plain"]) > 1e-3
    assert (d[big] / np.abs(vals["plain"][big])).max() < 1e-5


@pytest.mark.parametrize("nucleus", [(82, 208, 6.68, 0.447), (79, 197, 6.38, 0.535), (8, 16, 2.608, 0.513)])
def test_fast_gaa_table_fp32_integrands(ug, nucleus):
    """The fast form's G_AA spline (T_A and G_AA integrands in FP32, sums in
    FP64) against the plain path's FP64 one: within 2e-6 absolutely and 2e-5
    relative to values above 1e-3 (Pb-Pb measured 6.4e-7 and 6.9e-6, the
    relative figure where G_AA = exp(-sigma T_AA) ~ 1e-3 multiplies T_AA's
    error by sigma T_AA ~ 7; G_AA is in [0, 1] and the fast form's budget is
    1e-4)."""
    z, a_, r, d = nucleus
    b = np.linspace(0.0, 20.0, 2001)
    vals = {}
    for meth in ("plain", "fast"):
        g = ug.UpcGenerator(dict(C1, NUCLEUS_Z=z, NUCLEUS_A=a_, WS_R=r, WS_A=d, BINS_M=3, BINS_Y=3))
        g.setLumiMethod(meth)
        g.init()
        vals[meth] = g.nucProcessCS.spline("gaa", b)
    diff = np.abs(vals["fast"] - vals["plain"])
    big = np.abs(vals["plain"]) > 1e-3
    rel = diff[big] / np.abs(vals["plain"][big])
    print("G_AA fp32 integrands:", nucleus, "abs", diff.max(), "rel", rel.max())
    assert diff.max() < 2e-6
    assert rel.max() < 2e-5


def test_fast_form_factor_table(ug, oracle_mod):
    """The fast form's form-factor spline: its 65,536 knot values (the closed
    form with one sincos and sinh/cosh from one exp) against the oracle's
    calcFormFac within 2e-9 of F(0) (the plain path's bound: at the smallest
    Q^2 the closed form cancels to O(Q^4) and the device's and the host's
    last-bit sin/cos/sinh/cosh differences reach ~1e-9 of F); between the
    knots within 1e-12 of F(0)
    above Q^2 = 1e-3 GeV^2, and within 1e-6 of F(0) in the first intervals,
    where the natural spline's free end (second derivative 0 at Q2min)
    departs from F (5.4e-7 measured for a natural spline on these knots)."""
    p = dict(C1, FLUX_POINT=0, BINS_M=3, BINS_Y=3)
    g = ug.UpcGenerator(p)
    g.setLumiMethod("fast")
    g.init()
    o = oracle_mod.Oracle(p, threads=os.cpu_count())
    o.init_tables()
    n, q2min, q2max = 65536, 1e-9, 2.0
    h = (q2max - q2min) / n
    knots = q2min + h * np.concatenate([np.arange(0, 64), np.arange(64, n - 1, 97)])
    f0 = abs(o.form_factor(q2min))
    at_knots = np.abs(g.nucProcessCS.spline("formfac", knots) -
                      np.array([o.form_factor(x) for x in knots])).max() / f0
    mid = np.linspace(1e-3, 1.999, 3001)
    between = np.abs(g.nucProcessCS.spline("formfac", mid) -
                     np.array([o.form_factor(x) for x in mid])).max() / f0
    first = np.geomspace(1e-9, 1e-3, 200)
    near0 = np.abs(g.nucProcessCS.spline("formfac", first) -
                   np.array([o.form_factor(x) for x in first])).max() / f0
    print("fast form factor / F(0): knots", at_knots, "above 1e-3", between, "first intervals", near0)
    assert at_knots < 2e-9
    assert between < 1e-12
    assert near0 < 1e-6


def test_fast_contraction_on_reference_fluxes(ug):
    """Method 2: the plain path's node fluxes (the reference's QAGS) through
    the projection and the tensor-core contraction -- isolates the
    contraction's error from the flux tables'."""
    p = dict(C1, PROC_ID=15, FLUX_POINT=0, BREAKUP_MODE=2, BINS_M=41, BINS_Y=25)
    out = {}
    for meth in ("plain", "hybrid"):
        g = ug.UpcGenerator(p)
        g.setLumiMethod(meth)
        g.init()
        out[meth] = g.lumiTable()
    rel = np.abs(out["hybrid"] / out["plain"] - 1)
    assert rel.max() < 2e-5, rel.max()


def test_grid_form_config3(ug, oracle_mod):
    """Luminosity method 3 (grid form, the precision form of the point-flux
    configuration with XnXn breakup): a 4096 x 2048 flux matrix, G on 2048
    radii in 1 .. 500 fm, L = N G N^T as two tensor-core products.  Its own
    quadrature differs from the reference's per-cell midpoint rule; measured on
    201 x 61: 1.7e-3 max / 6.1e-4 median relative on cells above 1e-5 of the
    maximum, 4.4e-4 on sigma_tot.  The bounds below state that difference."""
    p = dict(C1, BREAKUP_MODE=2)
    g = ug.UpcGenerator(p)
    g.setLumiMethod("grid")
    g.init()
    lumi = g.lumiTable()
    _, tot = g.nucCSYM()
    o = oracle_mod.Oracle(p, threads=os.cpu_count())
    o.init_tables()
    ref = o.lumi_table()
    _, rtot, _ = o.nuc_cs_ym(ref)
    big = np.abs(ref) >= 1e-5 * np.abs(ref).max()
    rel = np.abs(lumi / ref - 1)[big]
    assert rel.max() < 5e-3 and np.median(rel) < 1.5e-3, (rel.max(), np.median(rel))
    assert abs(tot / rtot - 1) < 1e-3
    assert g.timings()["contract_ms"] > 0


@pytest.mark.parametrize("params", [
    C1,
    dict(C1, PROC_ID=15, FLUX_POINT=0, BREAKUP_MODE=2, BINS_M=41, BINS_Y=25),
    dict(C1, PROC_ID=13, BREAKUP_MODE=2, USE_POLARIZED_CS=1, FLUX_POINT=0, BINS_M=21, BINS_Y=25),
], ids=["point-201x61", "form-xnxn", "form-polarized"])
@pytest.mark.parametrize("other", ["gather", "fused"])
def test_operand_paths_agree(ug, params, other):
    """The fast form's three operand paths on the same bf16 hi / lo operands and
    survival kernel: the default (both operands dense on the radial grid, A1
    through TMA, A2 read by the epilogue), "gather" (the A2 row-dot gathered at
    side 1's node stencils) and "fused" (A1 built in shared memory from the
    node lists).  The tables
    differ only by the FP32 summation order of the row-dot (<= 2e-6 relative
    on cells above 1e-12 of the maximum)."""
    out = {}
    pol = params.get("USE_POLARIZED_CS", 0)
    for meth in ("fast", other):
        g = ug.UpcGenerator(params)
        g.setLumiMethod(meth)
        g.init()
        out[meth] = g.lumiTable(polarized=bool(pol))
        out[meth + "_tot"] = g.nucCSYM()[1]
    pairs = zip(out["fast"], out[other]) if pol else [(out["fast"], out[other])]
    for a, b in pairs:
        big = np.abs(b) >= 1e-12 * np.abs(b).max()
        assert np.all((a == 0) == (b == 0))
        rel = np.abs(a[big] / b[big] - 1)
        assert rel.max() <= 2e-6, rel.max()
    assert abs(out["fast_tot"] / out[other + "_tot"] - 1) <= 1e-6


def test_grid_form_tf32_arm(ug, oracle_mod):
    """Luminosity method 7: the grid form with its two products on tcgen05
    kind::tf32 (FP32 operands, 10 mantissa bits kept, FP32 accumulation)
    instead of the three-term bf16 split.  It carries the grid form's own
    quadrature difference (as method 3) plus the TF32 rounding; both are
    stated here against the oracle, beside the bf16x3 arm on the same table."""
    p = dict(C1, BREAKUP_MODE=2)
    o = oracle_mod.Oracle(p, threads=os.cpu_count())
    o.init_tables()
    ref = o.lumi_table()
    big = np.abs(ref) >= 1e-5 * np.abs(ref).max()
    out = {}
    for meth in ("grid", "grid-tf32"):
        g = ug.UpcGenerator(p)
        g.setLumiMethod(meth)
        g.init()
        lumi = g.lumiTable()
        out[meth] = (np.abs(lumi / ref - 1)[big], g.nucCSYM()[1], g.timings()["contract_ms"])
    rel32, tot32, t32 = out["grid-tf32"]
    rel16, tot16, t16 = out["grid"]
    _, rtot, _ = o.nuc_cs_ym(ref)
    print(f"grid form vs oracle: bf16x3 max {rel16.max():.2e} median {np.median(rel16):.2e} "
          f"sigma {tot16 / rtot - 1:.2e} products {t16:.4f} ms; tf32 max {rel32.max():.2e} "
          f"median {np.median(rel32):.2e} sigma {tot32 / rtot - 1:.2e} products {t32:.4f} ms")
    assert rel32.max() < 1e-2 and np.median(rel32) < 3e-3, (rel32.max(), np.median(rel32))
    assert abs(tot32 / rtot - 1) < 2e-3
    # the TF32 rounding on top of the grid quadrature's difference
    assert np.median(rel32) < 3 * np.median(rel16) + 1e-3


def test_fast_flux_table_vs_converged_quadrature(ug, oracle_mod):
    """The Q(w, b) table of the fast form (256 Gauss-Legendre nodes on q <= 1.5
    GeV, three panels of them in ln q below 0.094 GeV, as a double-float
    product H J on the FP32 pipe, the clamped tail in closed form) against the
    oracle's fluxForm integrated to convergence, at table nodes with w < 0.05
    gamma (where the tail's closed form holds) and |Q| above 1e-3 of its
    row's largest: N = factor Q^2 / (A^2 k).  The node layout integrates to
    7e-7 of the converged integral at worst over these w and b (measured here
    5e-8 on the sampled nodes; uniform panels from q = 0 missed the
    integrand's turn-on at q ~ w / gamma by up to 1e-4 near b = 2R); the
    double-float product adds ~1e-13."""
    p = dict(C1, PROC_ID=15, FLUX_POINT=0, BREAKUP_MODE=2, BINS_M=21, BINS_Y=13)
    g = ug.UpcGenerator(p)
    g.setLumiMethod("fast")
    g.init()
    q, (lw0, hw, lb0, hb) = g.fastFluxTable()
    o = oracle_mod.Oracle(dict(p, ORACLE_FLUX_EPS=1e-10), threads=os.cpu_count())
    o.init_tables()
    gam = o.gamma()
    fac = 82 * 82 / 137.035999074 / np.pi ** 2 / 0.1973269718 ** 2
    rng = np.random.default_rng(5)
    rows = [i for i in range(512) if np.exp(lw0 + i * hw) < 0.05 * gam]
    worst = []
    for i in rng.choice(rows, 24, replace=False):
        k = float(np.exp(lw0 + i * hw))
        row = q[i]
        for j in rng.choice(256, 8, replace=False):
            if abs(row[j]) < 1e-3 * np.abs(row).max():
                continue
            b = float(np.exp(lb0 + j * hb))
            if b > 2 * 6.68:  # fluxForm takes the point flux beyond 2R
                continue
            qref = np.sqrt(o.flux_form(b, k) * 208 * 208 * k / fac)
            worst.append((abs(abs(row[j]) / qref - 1), i, j, k, b))
    print("Q table vs converged fluxForm: worst", max(worst))
    assert len(worst) > 100
    assert max(worst)[0] < 1e-6, max(worst)
