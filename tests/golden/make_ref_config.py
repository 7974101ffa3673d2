"""What the reference makes of parameters.in files (run once; results committed
as tests/golden/ref_config.json).

Each file is read by the reference's own configGeneratorFromFile
(src/UpcGenerator.cpp:318-346) and init (the process overrides, :57-181),
compiled from its sources by oracle/build.py (build_ref_gen,
oracle/ref_out_shim.cpp), one file per fresh process.  Stored per file: the
grid init ends with (m, y, z ranges and bins), PROC_ID, NEVENTS and the
output flags.  The files exercise the reader's rules and quirks: comment
lines, trailing comments, unknown keys, a key without a value (it takes the
previous line's value), an empty line, a line that starts with spaces and a
'#', the ALP mass window, the dilepton MMIN clamp.

Usage: python tests/golden/make_ref_config.py
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
OUT = os.path.join(HERE, "ref_config.json")

FILES = {
    "comments_and_unknown_keys": "# a comment line\nPROC_ID 15\nBINS_M 17   # trailing comment\n"
                                 "BINS_Y 9\nYMIN -2.5\nPYTHIA_VERSION 8\nSOME_UNKNOWN_KEY 42\n\n"
                                 "MMAX 20\nBINS_Z 10\nFLUX_POINT 1\n",
    "key_without_value": "PROC_ID 15\nBINS_M 11\nBINS_Y 7\nMMAX 30\nYMAX\nBINS_Z 12\nFLUX_POINT 1\n",
    "alp_window_and_output": "PROC_ID 51\nALP_MASS 2\nALP_WIDTH 0.05\nBINS_M 9\nBINS_Y 7\nBINS_Z 8\n"
                             "FLUX_POINT 1\nUSE_HEPMC_OUTPUT 1\nUSE_ROOT_OUTPUT 0\nNEVENTS 123\n",
    "muon_mmin_clamp": "PROC_ID 13\nMMIN 0.1\nMMAX 5\nBINS_M 9\nBINS_Y 7\nBINS_Z 8\nFLUX_POINT 1\n"
                       "DO_PT_CUT 1\nPT_MIN 0.5\nNON_ZERO_GAM_PT 0\n",
    "indented_comment_polarized": "  # indented comment\nPROC_ID 15\nBINS_M 9\nBINS_Y 7\nBINS_Z 8\n"
                                  "FLUX_POINT 1\nUSE_POLARIZED_CS 1\nBREAKUP_MODE 3\n"
                                  "ZMIN -0.5 extra tokens\nZMAX 0.75\n",
}
INT_NAMES = ["nm", "ny", "nz", "PROC_ID", "BREAKUP_MODE", "FLUX_POINT", "USE_POLARIZED_CS",
             "NON_ZERO_GAM_PT", "DO_PT_CUT", "DO_ETA_CUT", "USE_ROOT_OUTPUT", "USE_HEPMC_OUTPUT"]


def run_one(text):
    """The reference's reading of one file, in this process (call it in a
    fresh one)."""
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    so = ob.build_ref_gen()
    if so is None:
        raise RuntimeError("reference sources not present")
    L = C.CDLL(so)
    grid = np.zeros(6)
    ints = np.zeros(12, dtype=np.int32)
    nev = C.c_int64()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "parameters.in")
        with open(path, "w") as f:
            f.write(text)
        rc = L.uref_config_file(path.encode(), d.encode(), grid.ctypes.data_as(C.c_void_p),
                                ints.ctypes.data_as(C.c_void_p), C.byref(nev))
    if rc != 0:
        raise RuntimeError(f"uref_config_file failed: {rc}")
    out = dict(zip(["mmin", "mmax", "ymin", "ymax", "zmin", "zmax"], map(float, grid)))
    out.update(zip(INT_NAMES, map(int, ints)))
    out["NEVENTS"] = nev.value
    return out


def run_fresh(name):
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--one", name],
                       check=True, capture_output=True, text=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        print(json.dumps(run_one(FILES[sys.argv[2]])))
        return
    out = {name: {"text": text, "reference": run_fresh(name)} for name, text in FILES.items()}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
