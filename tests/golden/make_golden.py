"""Generate the golden fixtures of tests/golden/ (run once, results committed).

Two independent sources pin the C++ oracle:

* ``ref_elem.json`` -- values of the reference's *own* elementary gamma-gamma
  cross sections (src/UpcTwoPhotonDilep.cpp, src/UpcTwoPhotonALP.cpp compiled
  from the reference sources by oracle/build.py into oracle/_ref/).  These are
  the only reference translation units that build without ROOT/GSL.
* ``numpy_restatement.json`` -- a second, independent restatement of the
  luminosity path in numpy/scipy (this file): scipy.special.k0/k1/j1 for the
  Bessel functions, scipy.interpolate.CubicSpline(bc_type="natural") for GSL's
  natural cspline, scipy.integrate.quad (QUADPACK QAGS) for the form-factor
  flux, and vectorised restatements of src/UpcCrossSection.cpp:152-163
  (rho0), :364-414 (G_AA), :436-445 (form factor), :752-1019 (breakup) and
  :221-271 (luminosity cells).

Usage: python tests/golden/make_golden.py   (needs the reference sources for
ref_elem.json; about a minute).
"""
import json
import os
import sys

import numpy as np
from scipy import integrate, interpolate, special

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ALPHA = 1.0 / 137.035999074
HC = 0.1973269718
MPROT = 0.9382720813
W10 = np.array([0.2955242247147529, 0.2692667193099963, 0.2190863625159820,
                0.1494513491505806, 0.0666713443086881])
X10 = np.array([0.1488743389816312, 0.4333953941292472, 0.6794095682990244,
                0.8650633666889845, 0.9739065285171717])


def simpson(v, h):
    n = len(v)
    return (v[0] + v[n - 1] + 4.0 * v[1:n - 1:2].sum() + 2.0 * v[2:n - 1:2].sum()) * h / 3.0


class Nucleus:
    def __init__(self, Z=82, A=208, R=6.68, a=0.447, sqrts=5020.0):
        self.Z, self.A, self.R, self.a, self.sqrts = Z, A, R, a, sqrts
        self.g = sqrts / (2 * MPROT)
        self.factor = Z * Z * ALPHA / np.pi / np.pi / HC / HC
        r = np.arange(200) * (20.0 / 199.0)
        self.rho0 = A / simpson(r * r / (1 + np.exp((r - R) / a)), 20.0 / 199.0) / 4 / np.pi
        self._gaa()
        self._formfac()

    def _gaa(self):
        nb, db = 200, 20.0 / 199
        ssm = self.sqrts ** 2 / (2 * MPROT + 2.1206) ** 2
        csnn = 0.1 * (34.41 + 0.2720 * np.log(ssm) ** 2 + 13.07 * ssm ** -0.4473 - 7.394 * ssm ** -0.5486)
        b = np.arange(nb) * db
        rr = np.sqrt(b[:, None] ** 2 + b[None, :] ** 2)
        rho = self.rho0 / (1 + np.exp((rr - self.R) / self.a))
        ta = 2 * np.array([simpson(row, db) for row in rho])
        sta = interpolate.CubicSpline(b, ta, bc_type="natural")
        s = b
        cosk = np.cos(np.pi * X10)
        g = []
        for bi in b:
            r = np.sqrt(bi * bi + s[:, None] ** 2 + 2 * bi * s[:, None] * cosk[None, :])
            sum_phi = (2 * np.pi * W10[None, :] * sta(np.minimum(r, 20.0))).sum(axis=1)
            vs = 2 * s * sta(np.minimum(s, 20.0)) * sum_phi
            g.append(np.exp(-csnn * simpson(vs, db)))
        self.gaa = interpolate.CubicSpline(b, np.array(g), bc_type="natural")

    def form_factor(self, q2):
        q = np.sqrt(q2) / HC
        a, R, rho0 = self.a, self.R, self.rho0
        ff = 4 * np.pi ** 2 * rho0 * a ** 3 / ((q * a) ** 2 * np.sinh(np.pi * q * a) ** 2) * (
            np.pi * q * a * np.cosh(np.pi * q * a) * np.sin(q * R) - q * R * np.cos(q * R) * np.sinh(np.pi * q * a))
        return ff + 8 * np.pi * rho0 * a ** 3 * np.exp(-R / a) / (1 + (q * a) ** 2) ** 2

    def _formfac(self):
        n = 1000000
        dq = (2.0 - 1e-9) / n
        x = 1e-9 + np.arange(n) * dq
        self.ff = interpolate.CubicSpline(x, self.form_factor(x), bc_type="natural")
        self.q2clamp = 2.0 - dq

    def flux_point(self, b, k):
        x = b * k / self.g / HC
        k0 = np.where(x > 1e-10, special.k0(np.maximum(x, 1e-300)), 0.0)
        k1 = np.where(x > 1e-10, special.k1(np.maximum(x, 1e-300)), 0.0)
        return self.factor * k / self.g ** 2 * (k1 * k1 + k0 * k0 / self.g ** 2)

    def flux_form(self, b, k):
        if b > 2 * self.R:
            return float(self.flux_point(b, k))
        w2 = k * k / self.g / self.g

        def f(q):
            t = q * q + w2
            return q * q * float(self.ff(t if t < 2.0 else self.q2clamp)) / t * special.j1(b * q / HC)

        res = integrate.quad(f, 0.0, 10.0, epsabs=1e-4, epsrel=1e-4, limit=1000)[0]
        return self.factor * (res / self.A) ** 2 / k


# ----------------------------------------------------------- breakup ----
E1 = [103., 106., 112., 119., 127., 132., 145., 171., 199., 230., 235., 254., 280., 300., 320.,
      330., 333., 373., 390., 420., 426., 440.]
S1 = [12.0, 11.5, 12.0, 12.0, 12.0, 15.0, 17.0, 28.0, 33.0, 52.0, 60.0, 70.0, 76.0, 85.0, 86.0,
      89.0, 89.0, 75.0, 76.0, 69.0, 59.0, 61.0]
E2 = [2000., 3270., 4100., 4810., 6210., 6600., 7790., 8400., 9510., 13600., 16400.]
S2 = [.1266, .1080, .0805, .1017, .0942, .0844, .0841, .0755, .0827, .0626, .0740]
E3 = [26., 28., 30., 32., 34., 36., 38., 40., 44., 46., 48., 50., 52., 55., 57., 62., 64., 66.,
      69., 72., 74., 76., 79., 82., 86., 92., 98., 103.]
S3 = [30., 21.5, 22.5, 18.5, 17.5, 15., 14.5, 19., 17.5, 16., 14., 20., 16.5, 17.5, 17., 15.5,
      18., 15.5, 15.5, 15., 13.5, 18., 14.5, 15.5, 12.5, 13., 13., 12.]


def breakup_tables(g, sigt, sigtn):
    gt = 2 * g * g - 1
    zp, ap, si1, g1, o1, o0 = 82, 208, 640., 4.05, 13.42, 7.4
    scon = .1 * g1 * g1 * si1
    ne = int((25. - o0) / .05) + 1
    ee = [o0 + i * .05 for i in range(ne)]
    se = [scon * e * e / ((o1 * o1 - e * e) ** 2 + e * e * g1 * g1) for e in ee]
    for e, s in zip(E3[:27], S3[:27]):
        ee.append(e); se.append(.1 * ap * s / 208.)
    for e, s in zip(E1, S1):
        ee.append(e); se.append(.1 * ap * s / 208.)
    for j in range(9, 71):
        ee.append(ee[-1] + 25.); se.append(.1 * (zp * sigt[j] + (ap - zp) * sigtn[j]))
    for e, s in zip(E2, S2):
        ee.append(e); se.append(.1 * ap * s)
    s = .002 * .94 * ee[-1]
    for _ in range(150 if gt > 2 * 150 * 150 else 100):
        s *= 10 ** .05
        ee.append(1000. * .5 * (s - .94 * .94) / .94)
        se.append(.1 * .65 * ap * (.0677 * s ** .0808 + .129 * s ** (-.4525)))
    zcon = zp / (gt * 3.14159 * 197.3269718) * zp / (gt * 3.14159 * 197.3269718) / 137.04
    return np.array(ee), np.array(se), zcon, gt


def k1_as(x):
    x = np.asarray(x, dtype=float)
    y = x * x / 4
    u = (x / 3.75) ** 2
    i1 = x * (0.5 + u * (0.87890594 + u * (0.51498869 + u * (0.15084934 + u * (0.2658733e-1 + u * (0.301532e-2 + u * 0.32411e-3))))))
    small = np.log(np.minimum(x, 2) / 2) * i1 + (1 / x) * (1. + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 + y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))))
    yy = 2 / np.maximum(x, 1e-300)
    large = np.exp(-x) / np.sqrt(x) * (1.25331414 + yy * (0.23498619 + yy * (-0.3655620e-1 + yy * (0.1504268e-1 + yy * (-0.780353e-2 + yy * (0.325614e-2 + yy * (-0.68245e-3)))))))
    return np.where(x <= 2, small, large)


def breakup_prob(b, mode, g, tabs):
    ee, se, zcon, gt = tabs
    omaxx = 1e10 if g > 500 else 1e7
    out = []
    for bb in np.atleast_1d(b):
        omax = min(omaxx, 4 * gt * 197.3269718 / bb)
        if omax < 7.4:
            out.append(0.0)
            continue
        n = int(np.searchsorted(ee, omax, side="left"))  # ee[k] < omax for k < n
        kk = k1_as(ee[:n] * bb / (197.3269718 * gt))
        f = se[:n] * ee[:n] * kk * kk
        pxn = float(np.sum(zcon * np.diff(ee[:n]) * .5 * (f[:-1] + f[1:])))
        e = np.exp(-pxn)
        out.append({1: 1.0, 2: (1 - e) ** 2, 3: np.exp(-2 * pxn), 4: 2 * e * (1 - e)}[mode])
    return np.array(out)


def lumi_cell(nuc, M, Y, is_point, mode, brk_spline):
    k1, k2 = M / 2 * np.exp(Y), M / 2 * np.exp(-Y)
    bmin = nuc.R if is_point else 0.05 * nuc.R

    def grid(k):
        bmax = max(5 * nuc.g * HC / k, 5 * nuc.R)
        ld = (np.log(bmax) - np.log(bmin)) / 120
        i = np.arange(120)
        bl, bh = bmin * np.exp(i * ld), bmin * np.exp((i + 1) * ld)
        b = (bh + bl) / 2
        return b, b * (bh - bl)

    b1, w1 = grid(k1)
    b2, w2 = grid(k2)
    if is_point:
        f1, f2 = nuc.flux_point(b1, k1), nuc.flux_point(b2, k2)
    else:
        f1 = np.array([nuc.flux_form(b, k1) for b in b1])
        f2 = np.array([nuc.flux_form(b, k2) for b in b2])
    cosk = np.cos(np.pi * X10)
    bb = np.sqrt(b1[:, None, None] ** 2 + b2[None, :, None] ** 2 + 2 * b1[:, None, None] * b2[None, :, None] * cosk)
    brk = 1.0 if mode == 1 else brk_spline(np.minimum(bb, 20.0))
    gaa = np.where(bb < 20, nuc.gaa(np.minimum(bb, 20.0)), 1.0)
    sphi = (brk * gaa * W10).sum(axis=2)
    return float(2 * np.pi ** 2 * M * np.einsum("i,ij,j->", f1 * w1, sphi, f2 * w2))


def make_ref_elem():
    from oracle import oracle
    L = oracle.ref_lib()
    if L is None:
        print("reference sources not available; ref_elem.json not regenerated")
        return
    out = {"source": "reference src/UpcTwoPhotonDilep.cpp + src/UpcTwoPhotonALP.cpp compiled "
                     "by oracle/build.py", "dilep": [], "alp": []}
    rng = np.random.default_rng(2024)
    for pdg in (11, 13, 15):
        mpart = L.uref_dilep_mass(pdg)
        for alep in (0.0, 0.00116):
            for m in list(2 * mpart * (1 + np.geomspace(1e-4, 30, 6))) + [3.56, 50.0]:
                zs = [-0.99, -0.3, 0.0, 0.45, 0.999]
                out["dilep"].append({
                    "pdg": pdg, "alep": alep, "m": m,
                    "cs_m": [L.uref_dilep_cs_m(pdg, alep, m, f) for f in (0, 1, 2)],
                    "z": zs,
                    "cs_zm": [[L.uref_dilep_cs_zm(pdg, alep, z, m, f) for z in zs] for f in (0, 1, 2)]})
    for mass, width in ((1.0, 0.01), (5.0, 0.1)):
        for m in (mass - 0.01, mass, mass + 0.02):
            out["alp"].append({"mass": mass, "width": width, "m": m, "cs_m": L.uref_alp_cs_m(mass, width, m)})
    _ = rng
    with open(os.path.join(HERE, "ref_elem.json"), "w") as f:
        json.dump(out, f, indent=1)


def data_table(name):
    """A photo-neutron data table, read from the oracle source (one copy)."""
    import re
    src = open(os.path.join(ROOT, "oracle", "oracle_cs.cpp")).read()
    m = re.search(r"static const double %s\[\d+\] = \{(.*?)\};" % name, src, re.S)
    return [float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]


def main():
    make_ref_elem()
    SIGT, SIGTN = data_table("sigt"), data_table("sigtn")
    nuc = Nucleus()
    out = {"source": "independent numpy/scipy restatement (tests/golden/make_golden.py)",
           "nucleus": {"Z": 82, "A": 208, "R": 6.68, "a": 0.447, "sqrts": 5020.0}}
    out["rho0"] = nuc.rho0
    bg = np.array([0.0, 1.0, 5.0, 7.3, 10.0, 12.5, 15.0, 17.7, 19.9])
    out["gaa"] = {"b": bg.tolist(), "v": nuc.gaa(bg).tolist()}
    q2 = np.array([1e-8, 1e-6, 1e-4, 1e-3, 0.01, 0.05, 0.2, 0.7, 1.5, 1.99])
    out["form_factor"] = {"q2": q2.tolist(), "v": nuc.form_factor(q2).tolist(),
                          "spline": nuc.ff(q2).tolist()}
    kx = np.array([1e-9, 1e-4, 0.01, 0.5, 1.9, 2.0, 2.1, 7.5, 29.9, 30.1, 120.0, 690.0])
    out["bessel"] = {"x": kx.tolist(), "k0": special.k0(kx).tolist(), "k1": special.k1(kx).tolist()}
    tabs = breakup_tables(nuc.g, SIGT, SIGTN)
    bb = np.array([1e-5, 0.1, 1.0, 6.0, 13.0, 19.99, 20.0, 55.0, 400.0, 999.0])
    out["breakup"] = {"b": bb.tolist(), "modes": {m: breakup_prob(bb, m, nuc.g, tabs).tolist() for m in (2, 3, 4)}}
    # breakup spline, XNXN, knots up to 20 fm + 257 (as the oracle)
    db = (1000 - 1e-6) / 1000000
    nuse = int((20 - 1e-6) / db) + 257
    kb = 1e-6 + np.arange(nuse) * db
    brk = interpolate.CubicSpline(kb, breakup_prob(kb, 2, nuc.g, tabs), bc_type="natural")
    out["breakup_spline_xnxn"] = {"b": bb[bb <= 20].tolist(), "v": brk(bb[bb <= 20]).tolist()}
    cells = []
    for (M, Y) in ((3.56, 0.0), (10.0, -2.1), (45.0, 4.0), (20.0, -5.9)):
        cells.append({"flux_point": 1, "mode": 1, "M": M, "Y": Y, "L": lumi_cell(nuc, M, Y, True, 1, None)})
        cells.append({"flux_point": 1, "mode": 2, "M": M, "Y": Y, "L": lumi_cell(nuc, M, Y, True, 2, brk)})
    for (M, Y) in ((5.0, 0.5), (30.0, -3.0)):
        cells.append({"flux_point": 0, "mode": 2, "M": M, "Y": Y, "L": lumi_cell(nuc, M, Y, False, 2, brk)})
    out["lumi_cells"] = cells
    rng = np.random.default_rng(11)
    fl = []
    for _ in range(12):
        b = float(rng.uniform(0.34, 13.3))
        k = float(np.exp(rng.uniform(np.log(4.4e-3), np.log(50))))
        fl.append({"b": b, "k": k, "v": nuc.flux_form(b, k)})
    out["flux_form"] = fl
    with open(os.path.join(HERE, "numpy_restatement.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("written")


if __name__ == "__main__":
    main()
