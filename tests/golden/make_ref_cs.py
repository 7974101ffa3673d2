"""Golden values of the reference's own UpcCrossSection (run once, results
committed as tests/golden/ref_cs.json).

The reference's src/UpcCrossSection.cpp and its process classes are compiled
where they lie (oracle/build.py: build_ref_cs) against the GSL / ROOT
stand-ins of oracle/refshim/, whose luminosity-path calls -- GSL's natural
cubic spline, QAGS, the Bessel functions K0, K1, J1 and ROOT's
TMath::BesselK1 -- are the oracle's restated primitives (each pinned to scipy
in tests/test_oracle_pins.py).  The values below therefore come from the
reference's own code for everything around those calls: rho0 (calcWSRho,
:152-163), the G_AA spline (prepareGAA, :364-414), the form factor
(calcFormFac, :436-445), the point and form-factor fluxes (fluxPoint /
fluxForm, :166-218, QAGS at 1e-4), the breakup probability and its spline
(calcBreakupProb / prepareBreakupProb, :416-434, 752-1019), the two-photon
luminosity per cell (calcTwoPhotonLumi / calcTwoPhotonLumiPol, :221-335) and
the photonuclear flux (calcPhotonFlux, :700-722).

The configurations cover the point and the Woods-Saxon form-factor flux, the
four breakup modes, gamma below and above the reference's omaxx switch at 500
(sqrt(s) 200 GeV for Au), a light nucleus, and the polarized luminosity; the
cells include the grid's mass and rapidity edges.  The GPU tests compare the
plain path with these values; tests/test_oracle_pins.py the oracle.

Usage: python tests/golden/make_ref_cs.py   (needs the reference sources;
about two minutes: the reference builds its 10^6-knot splines single-threaded).
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

PB = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "MMIN": 3.56, "MMAX": 50, "BINS_M": 1001, "YMIN": -6, "YMAX": 6, "BINS_Y": 121}
CONFIGS = {
    "pb_point_mode1": dict(PB, FLUX_POINT=1, BREAKUP_MODE=1, PROC_ID=13),
    "pb_point_mode2": dict(PB, FLUX_POINT=1, BREAKUP_MODE=2, PROC_ID=13),
    "pb_point_mode3": dict(PB, FLUX_POINT=1, BREAKUP_MODE=3, PROC_ID=13),
    "pb_point_mode4": dict(PB, FLUX_POINT=1, BREAKUP_MODE=4, PROC_ID=13),
    "pb_form_mode2": dict(PB, FLUX_POINT=0, BREAKUP_MODE=2, PROC_ID=15),
    "pb_form_mode2_pol": dict(PB, FLUX_POINT=0, BREAKUP_MODE=2, PROC_ID=13, USE_POLARIZED_CS=1),
    "au200_form_mode4": dict(PB, NUCLEUS_Z=79, NUCLEUS_A=197, WS_R=6.38, WS_A=0.535, SQRTS=200,
                             FLUX_POINT=0, BREAKUP_MODE=4, PROC_ID=15, MMIN=1.0, MMAX=10.0,
                             BINS_M=201, YMIN=-3, YMAX=3, BINS_Y=61),
    "o16_form_mode3_alp": dict(PB, NUCLEUS_Z=8, NUCLEUS_A=16, WS_R=2.608, WS_A=0.513,
                               SQRTS=5360, FLUX_POINT=0, BREAKUP_MODE=3, PROC_ID=51,
                               ALP_MASS=1.0, ALP_WIDTH=0.01, MMIN=0.96, MMAX=1.04, BINS_M=201),
}
B_GAA = [0.0, 0.37, 1.5, 4.2, 6.68, 9.9, 13.3, 17.0, 19.95]
Q2 = [1e-9, 1e-4, 3e-3, 0.02, 0.1, 0.5, 1.3, 1.999]
BK = [(0.3, 0.02), (1.0, 0.5), (3.34, 2.5), (4.5545, 10.75), (6.0, 40.0), (12.0, 1.0),
      (13.3, 150.0), (20.0, 0.3), (60.0, 0.01)]
B_BRK = [1e-6, 0.5, 5.0, 10.0, 13.36, 15.0, 18.0, 19.99, 20.0]


def cells(p):
    """Left edges of the grid (prepareTwoPhotonLumi's cell values,
    src/UpcCrossSection.cpp:540-542): the first, middle and last mass rows,
    and rapidities at both edges, near the edges and in the middle."""
    nm, ny = p["BINS_M"], p["BINS_Y"]
    dm = (p["MMAX"] - p["MMIN"]) / nm
    dy = (p["YMAX"] - p["YMIN"]) / ny
    out = []
    for im in (0, 1, nm // 2, nm - 2, nm - 1):
        for iy in (0, 1, ny // 4, ny // 2, (3 * ny) // 4, ny - 2, ny - 1):
            out.append((im, iy, p["MMIN"] + dm * im, p["YMIN"] + dy * iy))
    return out


def one_config(name):
    """The values of one configuration, in a process of its own: the
    reference keeps process-wide state (the nucleus and splines, and
    calcBreakupProb's photo-neutron tables, built once per process for the
    Lorentz factor of its first call, src/UpcCrossSection.cpp:774-898)."""
    from oracle.oracle import RefCrossSection
    p = CONFIGS[name]
    r = RefCrossSection(p)
    e = {"params": p, "rho0": r.rho0()}
    e["gaa_spline"] = [[b, r.gaa_spline(b)] for b in B_GAA]
    e["form_factor"] = [[q2, r.form_factor(q2)] for q2 in Q2]
    e["flux_point"] = [[b, k, r.flux_point(b, k)] for b, k in BK]
    e["flux_form"] = [[b, k, r.flux_form(b, k)] for b, k in BK]
    mode = p["BREAKUP_MODE"]
    e["breakup_prob"] = [[b, r.breakup_prob(b, mode)] for b in B_BRK]
    if mode > 1:
        e["breakup_spline"] = [[b, r.breakup_spline(b)] for b in B_BRK]
    if p.get("USE_POLARIZED_CS"):
        e["lumi_pol"] = [[im, iy, m, y, *r.two_photon_lumi_pol(m, y)] for im, iy, m, y in cells(p)]
    else:
        e["lumi"] = [[im, iy, m, y, r.two_photon_lumi(m, y)] for im, iy, m, y in cells(p)]
    e["photon_flux"] = [[m, y, r.photon_flux(m, y)] for _, _, m, y in cells(p)[::5]]
    return name, e


def main():
    import concurrent.futures as cf
    import multiprocessing as mp

    from oracle.oracle import ref_cs_lib
    if ref_cs_lib() is None:
        print("reference sources not available; ref_cs.json not regenerated")
        return
    out = {"configs": {}}
    ctx = mp.get_context("spawn")
    with cf.ProcessPoolExecutor(max_workers=4, mp_context=ctx, max_tasks_per_child=1) as ex:
        for name, e in ex.map(one_config, list(CONFIGS)):
            print(name, flush=True)
            out["configs"][name] = e
    with open(os.path.join(HERE, "ref_cs.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote ref_cs.json")


if __name__ == "__main__":
    main()
