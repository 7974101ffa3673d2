"""Oracle luminosity tables of the full-grid Pb-Pb configuration (run once,
results committed as tests/golden/c2_lumi.npz).

Configuration: Pb-Pb (Z 82, A 208, R 6.68 fm, a 0.447 fm) at sqrt(s) = 5020
GeV, Woods-Saxon form-factor flux (FLUX_POINT 0), XnXn breakup (BREAKUP_MODE
2), m in [3.56, 50] GeV x 1001 bins, y in [-6, 6] x 121 bins: the table that
calcTwoPhotonLumi / prepareTwoPhotonLumi (src/UpcCrossSection.cpp:221-271,
463-592) build for it, L dm dy per cell, FP64.

Two tables come from the C++ oracle (oracle/oracle_cs.cpp, the line-by-line
restatement of those functions):

* ``ref``  -- the reference's own quadrature: fluxForm's QAGS at epsabs =
  epsrel = 1e-4 (src/UpcCrossSection.cpp:209-210), early stops included;
* ``conv`` -- the same cells with the form-factor flux integrated to
  convergence (oracle key ORACLE_FLUX_EPS = 1e-10; not a reference key).

Both are stored for every cell (121,121 each) together with the sigma_tot of
gamma gamma -> tau tau that calcNucCrossSectionYM (:594-698) folds from each.
Full tables take about 25 min (ref) and 100 min (conv) on 8 cores; the GPU
tests read the file only.

Usage: python tests/golden/make_c2_fixture.py [threads]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

C2 = {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
      "PROC_ID": 15, "LEP_A": 0, "FLUX_POINT": 0, "BREAKUP_MODE": 2,
      "MMIN": 3.56, "MMAX": 50, "BINS_M": 1001, "YMIN": -6, "YMAX": 6, "BINS_Y": 121,
      "ZMIN": -1, "ZMAX": 1, "BINS_Z": 100}
CONV_EPS = 1e-10
OUT = os.path.join(HERE, "c2_lumi.npz")


def table(params, threads, block=50):
    from oracle.oracle import Oracle
    o = Oracle(params, threads=threads)
    o.init_tables()
    nm = o.grid()["nm"]
    rows = []
    t0 = time.time()
    for a in range(0, nm, block):
        rows.append(o.lumi_table(a, min(nm, a + block)))
        print(f"  rows {a}..{min(nm, a + block)}  {time.time() - t0:.0f} s", flush=True)
    lumi = np.concatenate(rows)
    _, tot, _ = o.nuc_cs_ym(lumi)
    return lumi, tot


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    print("reference quadrature (QAGS 1e-4)")
    ref, tot_ref = table(C2, threads)
    print("converged quadrature")
    conv, tot_conv = table(dict(C2, ORACLE_FLUX_EPS=CONV_EPS), threads)
    np.savez_compressed(OUT, ref=ref, conv=conv, sigma_tot_ref=tot_ref, sigma_tot_conv=tot_conv,
                        conv_eps=CONV_EPS)
    print(f"wrote {OUT}: sigma_tot ref {tot_ref!r} mb, conv {tot_conv!r} mb")


if __name__ == "__main__":
    main()
