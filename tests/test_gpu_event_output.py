"""generateEvents with file output on the GPU: the HepMC3 file and the
particle column file hold exactly the events of upcg_generate_events for the
same seed (several device batches, the device batch of the next events
overlapping the file work of the last ones), with the rejected count and the
fiducial cross section of the reference's loop (src/UpcGenerator.cpp:834-926)."""
import numpy as np
import pytest

from upcgen_gb300 import event_output as eo

pytestmark = pytest.mark.gpu

C2S = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
       "PROC_ID": 15, "FLUX_POINT": 0, "BREAKUP_MODE": 2, "MMIN": 3.56, "MMAX": 50,
       "BINS_M": 21, "YMIN": -6, "YMAX": 6, "BINS_Y": 13, "SEED": 5,
       "DO_PT_CUT": 1, "PT_MIN": 1, "DO_ETA_CUT": 1, "ETA_MIN": -2.4, "ETA_MAX": 2.4}
ALP = dict(C2S, PROC_ID=51, ALP_MASS=1, ALP_WIDTH=0.01, DO_PT_CUT=0, DO_ETA_CUT=0, FLUX_POINT=1)

HEAD = "HepMC::Version 3.02.04\nHepMC::Asciiv3-START_EVENT_LISTING\n"
TAIL = "HepMC::Asciiv3-END_EVENT_LISTING\n"


def _pair(ug, params):
    a = ug.UpcGenerator(params)
    a.init()
    b = ug.UpcGenerator(params)
    b.init()
    return a, b


@pytest.mark.parametrize("params", [C2S, ALP], ids=["tau-cuts", "alp"])
def test_hepmc_file(ug, tmp_path, monkeypatch, params):
    monkeypatch.setenv("UPCG_OUTPUT_BATCH", "7000")
    g, ref = _pair(ug, params)
    n = 30000
    path = tmp_path / "events.hepmc"
    rej = g.writeEvents(path, n, "hepmc", threads=4)
    ev, rej_ref = ref.generateEvents(n)
    assert rej == rej_ref
    assert g.fidNuclX() == ref.fidNuclX()
    text = path.read_text()
    assert text == HEAD + ref.formatHepMC3(ev, 0) + TAIL
    events, rows = eo.read_hepmc3(text)
    assert [e[0] for e in events] == list(range(n))


@pytest.mark.parametrize("params", [C2S, ALP], ids=["tau-cuts", "alp"])
def test_column_file(ug, tmp_path, monkeypatch, params):
    monkeypatch.setenv("UPCG_OUTPUT_BATCH", "7000")
    g, ref = _pair(ug, params)
    n = 30001
    path = tmp_path / "events.cols"
    rej = g.writeEvents(path, n, "columns")
    ev, rej_ref = ref.generateEvents(n)
    assert rej == rej_ref
    c = eo.read_particle_columns(path)
    ppe = g.particlesPerEvent()
    assert len(c["px"]) == n * ppe
    assert np.array_equal(c["eventNumber"], np.repeat(np.arange(n), ppe))
    assert np.array_equal(c["particleID"], np.tile(np.arange(1, ppe + 1), n))
    p0 = ev["p0"].astype(np.float64)
    p1 = ev["p1"].astype(np.float64)
    if ppe == 3:
        mom = np.stack([p0 + p1, p0, p1], 1)
        pdg = np.tile([51, 22, 22], n)
        st = np.tile([23, 33, 33], n)
        mo = np.tile([0, 1, 1], n)
    else:
        mom = np.stack([p0, p1], 1)
        s1 = np.where(ev["sign"] > 0, 1, -1)
        pdg = np.stack([15 * s1, -15 * s1], 1).ravel()
        st = np.full(2 * n, 23)
        mo = np.zeros(2 * n, dtype=int)
    assert np.array_equal(c["pdgCode"], pdg)
    assert np.array_equal(c["statusID"], st) and np.array_equal(c["motherID"], mo)
    for k, name in enumerate(("px", "py", "pz", "e")):
        assert np.array_equal(c[name], mom[:, :, k].ravel())


def test_empty_and_bad_path(ug, tmp_path):
    g = ug.UpcGenerator(dict(C2S, BINS_M=5, BINS_Y=5))
    g.init()
    path = tmp_path / "e.hepmc"
    assert g.writeEvents(path, 0) == 0
    assert path.read_text() == HEAD + TAIL
    with pytest.raises(ug.UpcgError):
        g.writeEvents(tmp_path / "no" / "such" / "dir.hepmc", 10)


def test_pinned_out_buffer(ug):
    """generateEvents, lumiTable and nucCSYM into page-locked arrays
    (upcg_host_alloc) give what they give into pageable ones; an out of the
    wrong size or type is refused."""
    g, ref = _pair(ug, dict(C2S, BINS_M=51, BINS_Y=25))
    lum = ug.pinned_array((51, 25), np.float64)
    csh = ug.pinned_array((25, 51), np.float64)
    assert g.lumiTable(out=lum) is lum and np.array_equal(lum, ref.lumiTable())
    cs, tot = g.nucCSYM(out=csh)
    cs_ref, tot_ref = ref.nucCSYM()
    assert cs is csh and np.array_equal(cs, cs_ref) and tot == tot_ref
    with pytest.raises(ValueError):
        g.lumiTable(out=np.zeros((25, 51)))
    with pytest.raises(ValueError):
        g.nucCSYM(out=np.zeros((25, 51), dtype=np.float32))
    n = 20000
    buf = ug.pinned_array(n + 5, ug.EVENT_DTYPE)
    ev, rej = g.generateEvents(n, out=buf)
    ev_ref, rej_ref = ref.generateEvents(n)
    assert rej == rej_ref and ev.base is not None
    assert np.array_equal(buf[:n].view(np.uint8), ev_ref.view(np.uint8))
    with pytest.raises(ValueError):
        g.generateEvents(n + 6, out=buf)
    with pytest.raises(ValueError):
        g.generateEvents(10, out=np.zeros(10, dtype=np.float32))
    del ev, buf  # frees the page-locked block


@pytest.mark.parametrize("flags", [(1, 1), (0, 0)], ids=["both-files", "no-file"])
def test_generate_event_files(ug, tmp_path, monkeypatch, flags):
    """The reference's generateEvents() (src/UpcGenerator.cpp:834-926) from the
    parameter keys: with USE_HEPMC_OUTPUT and USE_ROOT_OUTPUT both files hold
    the events generateEvents(n) gives for the same seed (the candidate
    sequence is rewound between them); with neither the loop still runs, so
    fidNuclX, the rejected count and the next candidate match."""
    use_root, use_hepmc = flags
    monkeypatch.chdir(tmp_path)
    n = 1000
    params = dict(C2S, NEVENTS=n, USE_ROOT_OUTPUT=use_root, USE_HEPMC_OUTPUT=use_hepmc)
    g, ref = _pair(ug, params)
    rej = g.generateEventFiles()
    ev, rej_ref = ref.generateEvents(n)
    assert rej == rej_ref
    assert g.fidNuclX() == ref.fidNuclX()
    assert g.fidNuclX() == g.totNuclX() * n / (n + rej_ref)
    assert g.candidateOffset() == ref.candidateOffset()
    if use_hepmc:
        assert (tmp_path / "events.hepmc").read_text() == HEAD + ref.formatHepMC3(ev, 0) + TAIL
    if use_root:
        c = eo.read_particle_columns(tmp_path / "events.cols")
        p0 = ev["p0"].astype(np.float64)
        assert np.array_equal(c["px"][0::2], p0[:, 0]) and np.array_equal(c["e"][0::2], p0[:, 3])
    if not use_root and not use_hepmc:
        assert not (tmp_path / "events.hepmc").exists() and not (tmp_path / "events.cols").exists()
