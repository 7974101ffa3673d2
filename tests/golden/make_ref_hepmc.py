"""The reference's HepMC3 text for seeded event records (run once; the SHA-256
and size of each text are committed as tests/golden/ref_hepmc.json).

The records are random event records of the library's layout (FP32 m, y, z,
sign and two 4-momenta), made by ``records()`` from a fixed seed.  Their
particle lists are the library's (UpcGenerator.particlesOf: generateEvent's
pdg codes, status codes, mothers and momenta), and they are written by the
reference's own writeEvent and WriterHepMC (src/UpcGenerator.cpp:589-628,
include/UpcGenerator.h:192-242), compiled here by oracle/build.py
(build_ref_gen, oracle/ref_out_shim.cpp).  The library's HepMC3 output of the
same records must be the same text, byte for byte.

Usage: python tests/golden/make_ref_hepmc.py
"""
import ctypes as C
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_hepmc.json")
# (PROC_ID, records, seed, number of the first event)
CASES = {"mumu": (13, 4000, 101, 17), "tautau": (15, 4000, 102, 0), "alp": (51, 4000, 103, 5)}


def records(event_dtype, n, seed):
    """Seeded records spanning 16 decades of momentum, both charge orders and
    a negative zero."""
    rng = np.random.default_rng(seed)
    ev = np.zeros(n, dtype=event_dtype)
    ev["m"] = rng.uniform(4, 50, n)
    ev["y"] = rng.uniform(-6, 6, n)
    ev["z"] = rng.uniform(-1, 1, n)
    ev["sign"] = rng.choice([-1.0, 1.0], n)
    for k in ("p0", "p1"):
        p = rng.normal(0, 10, (n, 3)) * np.exp(rng.uniform(-8, 8, (n, 1)))
        ev[k][:, :3] = p
        ev[k][:, 3] = np.sqrt((p.astype(np.float32).astype(np.float64) ** 2).sum(1) + 0.011)
    ev["p0"][0, 0] = -0.0
    return ev


def particle_arrays(gen, ev):
    """The library's particle lists of the records as arrays (pdg, status,
    mother [n][ppe], p4 [n][ppe][4])."""
    ppe = gen.particlesPerEvent()
    n = len(ev)
    pdg = np.zeros((n, ppe), dtype=np.int32)
    st = np.zeros_like(pdg)
    mo = np.zeros_like(pdg)
    p4 = np.zeros((n, ppe, 4))
    for i in range(n):
        for k, (a, b, c, p) in enumerate(gen.particlesOf(ev[i])):
            pdg[i, k], st[i, k], mo[i, k], p4[i, k] = a, b, c, p
    return ppe, pdg, st, mo, p4


def reference_text(ppe, pdg, st, mo, p4, first):
    """The HepMC3 file the reference's writer makes of these particle lists."""
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    so = ob.build_ref_gen()
    if so is None:
        raise RuntimeError("reference sources not present")
    L = C.CDLL(so)
    arrs = [np.ascontiguousarray(a) for a in (pdg, st, mo, p4)]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "events.hepmc")
        rc = L.uref_write_hepmc(path.encode(), C.c_int64(len(pdg)), ppe,
                                *[a.ctypes.data_as(C.c_void_p) for a in arrs], C.c_int64(first))
        if rc != 0:
            raise RuntimeError(f"uref_write_hepmc failed: {rc}")
        with open(path, "rb") as f:
            return f.read()


def main():
    sys.path.insert(0, ROOT)
    import upcgen_gb300 as ug
    out = {}
    for name, (proc, n, seed, first) in CASES.items():
        g = ug.UpcGenerator({"PROC_ID": proc})
        ev = records(ug.EVENT_DTYPE, n, seed)
        text = reference_text(*particle_arrays(g, ev), first)
        out[name] = {"proc": proc, "records": n, "seed": seed, "first_event": first,
                     "bytes": len(text), "sha256": hashlib.sha256(text).hexdigest()}
        print(name, out[name])
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
