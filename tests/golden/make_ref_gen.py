"""Events of the reference's own generator (run once, results committed as
tests/golden/ref_gen.npz).

oracle/build.py (build_ref_gen) compiles the reference's src/UpcGenerator.cpp,
src/UpcCrossSection.cpp and the process classes where they lie, against the
GSL / ROOT stand-ins of oracle/refshim/, into oracle/_ref/libupcref_gen.so;
oracle/ref_gen_shim.cpp runs UpcGenerator::init and the generateEvent loop
of generateEvents (src/UpcGenerator.cpp:57-181, 630-889) for one
configuration.  Each configuration runs in a fresh process (the reference
keeps its nucleus, splines and breakup tables as process globals) with one
luminosity thread, and its first N accepted events are stored: the pdg
codes, status codes, mothers and 4-momenta of generateEvent's particle lists,
the rejected count and totNuclX.

The configurations cover the event loop's branches: lepton pairs with and
without photon pT (NON_ZERO_GAM_PT), the pT and eta cuts (rejections), the
breakup modes, the point and the form-factor flux, the polarized cross
section (scalar / pseudoscalar z samplers) and the ALP (single particle and
uniform two-photon decay).

Usage: python tests/golden/make_ref_gen.py
"""
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_gen.npz")
N_EVENTS = 300
MAX_PARTICLES = 3

PB = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020}
CONFIGS = {
    "mumu_point": dict(PB, PROC_ID=13, LEP_A=0, FLUX_POINT=1, BREAKUP_MODE=1, MMIN=3.56, MMAX=50,
                       BINS_M=21, YMIN=-6, YMAX=6, BINS_Y=13, ZMIN=-1, ZMAX=1, BINS_Z=100, SEED=1,
                       NON_ZERO_GAM_PT=0),
    "tautau_cuts_xnxn": dict(PB, PROC_ID=15, LEP_A=0, FLUX_POINT=1, BREAKUP_MODE=2, MMIN=3.56,
                             MMAX=50, BINS_M=21, YMIN=-6, YMAX=6, BINS_Y=13, ZMIN=-1, ZMAX=1,
                             BINS_Z=100, SEED=7, NON_ZERO_GAM_PT=1, DO_PT_CUT=1, PT_MIN=1,
                             DO_ETA_CUT=1, ETA_MIN=-2.4, ETA_MAX=2.4),
    "mumu_formfactor_eta": dict(PB, PROC_ID=13, LEP_A=0, FLUX_POINT=0, BREAKUP_MODE=4, MMIN=3.56,
                                MMAX=50, BINS_M=9, YMIN=-4, YMAX=4, BINS_Y=7, ZMIN=-1, ZMAX=1,
                                BINS_Z=100, SEED=5, NON_ZERO_GAM_PT=1, DO_ETA_CUT=1,
                                ETA_MIN=-2.4, ETA_MAX=2.4),
    "tautau_polarized": dict(PB, PROC_ID=15, LEP_A=0, FLUX_POINT=1, BREAKUP_MODE=1, MMIN=3.56,
                             MMAX=8, BINS_M=11, YMIN=-3, YMAX=3, BINS_Y=7, ZMIN=-1, ZMAX=1,
                             BINS_Z=50, SEED=11, NON_ZERO_GAM_PT=0, USE_POLARIZED_CS=1),
    "alp_mode3": dict(PB, PROC_ID=51, ALP_MASS=1, ALP_WIDTH=0.01, FLUX_POINT=1, BREAKUP_MODE=3,
                      BINS_M=21, YMIN=-6, YMAX=6, BINS_Y=13, SEED=3, NON_ZERO_GAM_PT=1),
}


def run_one(params, n=N_EVENTS, threads=1):
    """The reference's events for one configuration, in this process (call it
    in a fresh one).  Returns (pdg, status, mother [n][3], p4 [n][3][4],
    rejected, tot_mb)."""
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    so = ob.build_ref_gen()
    if so is None:
        raise RuntimeError("reference sources not present")
    L = C.CDLL(so)
    keys = [k.encode() for k in params]
    vals = [str(v).encode() for v in params.values()]
    K = (C.c_char_p * len(keys))(*keys)
    V = (C.c_char_p * len(vals))(*vals)
    pdg = np.zeros((n, MAX_PARTICLES), dtype=np.int32)
    status = np.zeros_like(pdg)
    mother = np.zeros_like(pdg)
    p4 = np.zeros((n, MAX_PARTICLES, 4))
    rej, tot = C.c_int64(), C.c_double()
    with tempfile.TemporaryDirectory() as d:  # the reference's lock file goes here
        rc = L.uref_gen_run(K, V, len(keys), d.encode(), threads, C.c_int64(n), MAX_PARTICLES,
                            pdg.ctypes.data_as(C.c_void_p), status.ctypes.data_as(C.c_void_p),
                            mother.ctypes.data_as(C.c_void_p), p4.ctypes.data_as(C.c_void_p),
                            C.byref(rej), C.byref(tot))
    if rc != 0:
        raise RuntimeError(f"uref_gen_run failed: {rc}")
    return pdg, status, mother, p4, rej.value, tot.value


def run_fresh(name, out_path, n=N_EVENTS):
    """run_one for CONFIGS[name] in a fresh Python process; its arrays in out_path."""
    subprocess.run([sys.executable, os.path.abspath(__file__), "--one", name, out_path, str(n)],
                   check=True)
    d = np.load(out_path)
    return d["pdg"], d["status"], d["mother"], d["p4"], int(d["rejected"]), float(d["tot"])


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        name, path, n = sys.argv[2], sys.argv[3], int(sys.argv[4])
        pdg, status, mother, p4, rej, tot = run_one(CONFIGS[name], n)
        np.savez(path, pdg=pdg, status=status, mother=mother, p4=p4, rejected=rej, tot=tot)
        return
    arrays = {}
    with tempfile.TemporaryDirectory() as d:
        for name in CONFIGS:
            pdg, status, mother, p4, rej, tot = run_fresh(name, os.path.join(d, name + ".npz"))
            arrays[name + "/pdg"] = pdg
            arrays[name + "/status"] = status
            arrays[name + "/mother"] = mother
            arrays[name + "/p4"] = p4
            arrays[name + "/rejected"] = np.int64(rej)
            arrays[name + "/tot"] = np.float64(tot)
            print(f"{name}: {len(pdg)} events, {rej} rejected, totNuclX {tot!r} mb")
    arrays["configs"] = np.array(json.dumps(CONFIGS))
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
