"""Batched scans: several configurations with uneven grids through one
persistent tensor-core contraction inside a captured CUDA graph must give the
tables each configuration gets on its own, on the first run and on replays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NUCLEI = [(82, 208, 6.68, 0.447), (8, 16, 2.608, 0.513)]


def configs():
    out = []
    bins = [41, 61, 81]
    k = 0
    for z, a, r, d in NUCLEI:
        for mode in (1, 2, 4):
            out.append({"NUCLEUS_Z": z, "NUCLEUS_A": a, "WS_R": r, "WS_A": d,
                        "SQRTS": 5360 if k % 2 else 200, "PROC_ID": 51, "ALP_MASS": 1,
                        "ALP_WIDTH": 0.01, "BREAKUP_MODE": mode, "BINS_M": bins[k % 3],
                        "BINS_Y": 25, "YMIN": -5, "YMAX": 5, "SEED": 5 + k})
            k += 1
    return out


def test_scan_equals_single_configurations(ug):
    cfgs = configs()
    gens = [ug.UpcGenerator(c) for c in cfgs]
    scan = ug.Scan(gens)
    scan.run()
    first = [g.lumiTable() for g in gens]
    tots = [g.totNuclX() for g in gens]
    scan.run()  # graph replay
    info = scan.info()
    assert info["items"] > 0
    for i, c in enumerate(cfgs):
        again = gens[i].lumiTable()
        assert np.array_equal(again, first[i])
        single = ug.UpcGenerator(c)
        single.setLumiMethod("fast")
        single.init()
        ref = single.lumiTable()
        big = np.abs(ref) >= 1e-9 * np.abs(ref).max()
        rel = np.abs(first[i] / ref - 1)[big]
        assert rel.max() < 1e-5, (i, rel.max())
        assert tots[i] == pytest.approx(single.totNuclX(), rel=1e-5)
    ev, rej = gens[2].generateEvents(10000)
    assert len(ev) == 10000 and rej == 0  # ALP, no cuts
    assert np.all((ev["m"] >= 0.96) & (ev["m"] <= 1.04))


C5_NUCLEI = [(82, 208, 6.68, 0.447), (79, 197, 6.38, 0.535), (54, 129, 5.36, 0.59),
             (8, 16, 2.608, 0.513)]


@pytest.mark.parametrize("flux_point", [1, 0])
def test_scan_vs_oracle_per_nucleus(ug, oracle_mod, flux_point):
    """One scan over the four nuclei of the 64-configuration ALP scan (Pb, Au,
    Xe, O; sqrt(s) 200 and 5360 GeV; breakup modes 1-4; uneven grids), each
    table against the oracle: <= 1e-4 on cells above 1e-5 of the table's
    maximum and on sigma_tot.  With the form-factor flux the oracle integrates
    the flux to convergence (the fast form's contract)."""
    import os
    cfgs = []
    for k, (z, a, r, d) in enumerate(C5_NUCLEI):
        cfgs.append({"NUCLEUS_Z": z, "NUCLEUS_A": a, "WS_R": r, "WS_A": d,
                     "SQRTS": (200, 5360)[k % 2], "PROC_ID": 51, "ALP_MASS": 1,
                     "ALP_WIDTH": 0.01, "BREAKUP_MODE": 1 + k, "BINS_M": (11, 21)[k % 2],
                     "BINS_Y": 25, "FLUX_POINT": flux_point, "SEED": 3 + k})
    gens = [ug.UpcGenerator(c) for c in cfgs]
    scan = ug.Scan(gens)
    scan.run()
    for g, c in zip(gens, cfgs):
        lumi = g.lumiTable()
        oc = dict(c) if flux_point else dict(c, ORACLE_FLUX_EPS=1e-10)
        o = oracle_mod.Oracle(oc, threads=os.cpu_count())
        o.init_tables()
        ref = o.lumi_table()
        big = np.abs(ref) >= 1e-5 * np.abs(ref).max()
        rel = np.abs(lumi / ref - 1)[big]
        assert rel.max() < 1e-4, (c["NUCLEUS_Z"], rel.max())
        _, rtot, _ = o.nuc_cs_ym(ref)
        assert abs(g.totNuclX() / rtot - 1) < 1e-4, c["NUCLEUS_Z"]
