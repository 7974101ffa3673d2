"""The oracle's event loop pinned to the reference's own generator (no GPU).

tests/golden/ref_gen.npz (tests/golden/make_ref_gen.py) holds the first
accepted events of the reference's src/UpcGenerator.cpp, compiled where it
lies against the GSL / ROOT stand-ins of oracle/refshim/ (whose random
engines, histogram samplers and vector algebra are the oracle's own,
oracle/oracle_gen_prims.hpp), for five configurations: lepton pairs with and
without photon pT, pT and eta cuts, breakup modes 1-4, point and form-factor
flux, the polarized cross section, the ALP.  The oracle must reproduce them
bit for bit -- every 4-momentum, every pdg code and charge order, the
rejected count and totNuclX -- which pins its restatement of the samplers
(include/UpcSampler.h), generateEvent / generateEvents
(src/UpcGenerator.cpp:715-889), getPairMomentum / getPhotonPt
(src/UpcCrossSection.cpp:1021-1074) and the decays to the reference's code,
draw order included.  (GCC evaluates the reference's two gsl_rng_uniform
arguments of the 2-D sampler right to left; the pin is what showed it.)
The same events also pin the library's particle lists (getParticles,
particlesOf): pdg codes, charge order, status codes and mothers as the
reference's generateEvent makes them.
"""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = np.load(os.path.join(HERE, "golden", "ref_gen.npz"))
CONFIGS = json.loads(str(FIX["configs"]))


def _oracle_events(oracle_mod, params, n):
    o = oracle_mod.Oracle(params, threads=os.cpu_count() or 1)
    o.init_tables()
    pol = bool(params.get("USE_POLARIZED_CS", 0))
    if pol:
        l1, l2 = o.lumi_table(polarized=True)
    else:
        l1, l2 = o.lumi_table(), None
    o.set_threads(1)  # the reference ran its fold on one thread (sigma_tot's sum order)
    cs, tot, ratio = o.nuc_cs_ym(l1, l2)
    zm = np.concatenate([o.cs_zm_table(1), o.cs_zm_table(2)]) if pol else o.cs_zm_table(0)
    rec, rej, _ = o.generate(cs, zm, n, int(params["SEED"]), ratio=ratio if pol else None)
    return rec, rej, tot


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_oracle_events_bit_exact_vs_reference_generator(oracle_mod, name):
    params = CONFIGS[name]
    pdg, p4 = FIX[name + "/pdg"], FIX[name + "/p4"]
    rec, rej, tot = _oracle_events(oracle_mod, params, len(pdg))
    assert tot == float(FIX[name + "/tot"])
    assert rej == int(FIX[name + "/rejected"])
    proc = int(params["PROC_ID"])
    if proc == 51:
        # the ALP (particle 1) and its two photons from the uniform decay
        assert np.all(pdg == np.array([51, 22, 22]))
        d0, d1 = p4[:, 1], p4[:, 2]
    else:
        # the lepton pair, charges ordered by gRandom (sign of particle 1)
        s = rec[:, 3].astype(np.int32)
        assert np.array_equal(pdg[:, 0], s * proc) and np.array_equal(pdg[:, 1], -s * proc)
        assert np.all(pdg[:, 2] == 0)
        d0, d1 = p4[:, 0], p4[:, 1]
    assert np.array_equal(rec[:, 4:8], d0), np.argmax(np.any(rec[:, 4:8] != d0, axis=1))
    assert np.array_equal(rec[:, 8:12], d1)


def test_live_reference_generator():
    """When the reference sources are present: the generator rebuilt from them
    gives the committed events (the fixture is the reference, not a stale
    copy)."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_gen import CONFIGS as SRC_CONFIGS, run_fresh

    from oracle import build as ob
    if ob.build_ref_gen() is None:
        pytest.skip("reference sources not present")
    assert SRC_CONFIGS == CONFIGS
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        pdg, st, mo, p4, rej, tot = run_fresh("tautau_cuts_xnxn", os.path.join(d, "o.npz"), n=100)
    name = "tautau_cuts_xnxn"
    assert np.array_equal(pdg, FIX[name + "/pdg"][:100])
    assert np.array_equal(st, FIX[name + "/status"][:100])
    assert np.array_equal(mo, FIX[name + "/mother"][:100])
    assert np.array_equal(p4, FIX[name + "/p4"][:100])
    assert tot == float(FIX[name + "/tot"])


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_library_particle_lists_match_reference_generator(ug, name):
    """The drop-in's particle lists (getParticles / particlesOf, and the C++
    facade's generateEvent, which builds the same lists) against the
    reference's own generateEvent on its events: pdg codes with the charge
    order, status codes and mothers exactly; the momenta are the record's
    FP32 values; an ALP's own momentum is the sum of its photons'."""
    params = CONFIGS[name]
    pdg, st, mo, p4 = (FIX[name + "/" + k] for k in ("pdg", "status", "mother", "p4"))
    g = ug.UpcGenerator(params)
    ppe = g.particlesPerEvent()
    proc = int(params["PROC_ID"])
    rec = np.zeros(len(pdg), dtype=ug.EVENT_DTYPE)
    if proc == 51:
        rec["p0"], rec["p1"], rec["sign"] = p4[:, 1], p4[:, 2], 1.0
    else:
        rec["p0"], rec["p1"] = p4[:, 0], p4[:, 1]
        rec["sign"] = np.sign(pdg[:, 0] * proc)
    for k in range(len(rec)):
        got = g.particlesOf(rec[k])
        assert [q[0] for q in got] == list(pdg[k, :ppe]), k
        assert [q[1] for q in got] == list(st[k, :ppe]), k
        assert [q[2] for q in got] == list(mo[k, :ppe]), k
        first = 1 if proc == 51 else 0
        for i in range(first, ppe):
            assert got[i][3] == tuple(float(x) for x in p4[k, i].astype(np.float32)), (k, i)
        if proc == 51:
            assert np.allclose(got[0][3], p4[k, 0], rtol=0, atol=2e-6 * p4[k, 0, 3]), k


def test_sampler_bins_bit_exact_vs_reference_source(oracle_mod):
    """The oracle's getBinX / getBinY (the restatement the GPU's bin test is
    held to, tests/test_gpu_parity.py) against the reference's own
    UpcSampler2D functions compiled from include/UpcSampler.h
    (tests/golden/make_ref_bins.py): every bin edge, every step of the
    truncated numerator and 1-2 ulps around each, on the 201 x 61, 1001 x 121
    and 21 x 13 tau-pair grids, both axes -- including the index n the
    reference returns an ulp below the top edge."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_ref_bins as mb
    fix = np.load(os.path.join(HERE, "golden", "ref_bins.npz"))
    from oracle import build as ob
    live = ob.build_ref_gen() is not None
    for nm, ny in mb.GRIDS:
        em, ey = mb.edges(mb.MMIN, mb.MMAX, nm), mb.edges(mb.YMIN, mb.YMAX, ny)
        for axis, name, e, n in ((1, "m", em, nm), (0, "y", ey, ny)):
            x = mb.edge_values(e, n)
            ref = fix[f"{nm}x{ny}/{name}/bin"].astype(np.int32)
            assert len(ref) == len(x)
            if live:
                assert np.array_equal(mb.reference_bins(em, ey, x, axis), ref)
            got = np.array([oracle_mod.sampler_bin(n, e[0], e[-1], float(v)) for v in x])
            assert np.array_equal(got, ref), (nm, ny, name, np.flatnonzero(got != ref)[:5])
