"""The reference's getBinX / getBinY at every bin edge (run once; the bins
are committed as tests/golden/ref_bins.npz, the values they belong to are
remade by edge_values()).

UpcSampler2D::getBinX / getBinY (include/UpcSampler.h:124-134) compute
int(int(n (x - x0)) / (x1 - x0)): the int() truncates the numerator first, a
quirk that moves some values into the next-lower bin.  This script evaluates
the reference's own functions, compiled from its sources by oracle/build.py
(build_ref_gen, oracle/ref_gen_shim.cpp), on the sampler as
computeNuclXsection builds it (src/UpcGenerator.cpp:677-700: edges
lo + d i), for three grids of the tau-pair configuration, at every bin edge,
every step of the truncated numerator (lo + k / n) and 1-2 ulps on both
sides of each.

Usage: python tests/golden/make_ref_bins.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_bins.npz")
# (nm, ny) grids with m in [3.56, 50] GeV, y in [-6, 6]
GRIDS = [(201, 61), (1001, 121), (21, 13)]
MMIN, MMAX, YMIN, YMAX = 3.56, 50.0, -6.0, 6.0


def edges(lo, hi, n):
    """binEdges[i] = lo + d i, d = (hi - lo) / n (src/UpcGenerator.cpp:677-684)."""
    d = (hi - lo) / n
    return np.array([lo + d * i for i in range(n + 1)])


def edge_values(e, n):
    """The edges, the points lo + k / n where int(n (x - lo)) steps, and 1 and
    2 ulps on both sides of each, inside [lo, hi]."""
    lo, hi = e[0], e[-1]
    k_max = int(n * (hi - lo)) + 1
    base = np.concatenate([e, lo + np.arange(k_max + 1) / n])
    vals = [base]
    for direction in (np.inf, -np.inf):
        x = base
        for _ in range(2):
            x = np.nextafter(x, direction)
            vals.append(x)
    v = np.unique(np.concatenate(vals))
    return v[(v >= lo) & (v <= hi)]


def reference_bins(em, ey, x, axis):
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    so = ob.build_ref_gen()
    if so is None:
        raise RuntimeError("reference sources not present")
    L = C.CDLL(so)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(len(x), dtype=np.int32)
    ex = np.ascontiguousarray(ey)  # x axis of the sampler: rapidity
    eyy = np.ascontiguousarray(em)  # y axis: mass
    rc = L.uref_sampler_bins(len(ex) - 1, ex.ctypes.data_as(C.c_void_p), len(eyy) - 1,
                             eyy.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p),
                             C.c_int64(len(x)), axis, out.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise RuntimeError("uref_sampler_bins failed")
    return out


def main():
    arrays = {}
    for nm, ny in GRIDS:
        em, ey = edges(MMIN, MMAX, nm), edges(YMIN, YMAX, ny)
        for axis, name, e, n in ((1, "m", em, nm), (0, "y", ey, ny)):
            x = edge_values(e, n)
            arrays[f"{nm}x{ny}/{name}/bin"] = reference_bins(em, ey, x, axis).astype(np.int16)
            print(nm, ny, name, len(x))
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
