"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles the FP64 C++/OpenMP restatement in this folder
  into ``oracle/_build/libupcg_oracle.so``.
* ``build_ref()`` compiles the two translation units of the reference that build
  without ROOT/GSL -- ``src/UpcTwoPhotonDilep.cpp`` and ``src/UpcTwoPhotonALP.cpp``
  -- together with ``ref_shim.cpp`` into ``oracle/_ref/libupcref_elem.so``, when
  the reference sources are present.
* ``build_ref_cs()`` compiles the reference's ``src/UpcCrossSection.cpp`` and the
  process classes it creates (``UpcTwoPhotonDilep``, ``UpcTwoPhotonALP``,
  ``UpcTwoPhotonDipion``, ``UpcTwoPhotonLbyL``, ``UpcPhotoNuclearVM``) where they
  lie, against the GSL / ROOT stand-ins of ``refshim/`` (whose luminosity-path
  calls are the oracle's own restated primitives), with ``ref_cs_shim.cpp``
  into ``oracle/_ref/libupcref_cs.so``.  This pins the oracle's restatement of
  calcTwoPhotonLumi, fluxForm, calcBreakupProb, prepareGAA, calcPhotonFlux ...
  to the reference's own source text.
* ``build_ref_gen()`` adds the reference's ``src/UpcGenerator.cpp`` to those
  units, with ``ref_gen_shim.cpp``, into ``oracle/_ref/libupcref_gen.so``: the
  reference's own init and event loop, which pin the oracle's samplers and
  event generation.

``-ffp-contract=off`` keeps the x86 and aarch64 builds bit-identical (gcc
contracts a*b+c into FMAs by default on aarch64).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libupcg_oracle.so")
REF_SO = os.path.join(REF_DIR, "libupcref_elem.so")
REFERENCE_ROOT = os.environ.get("UPCG_REFERENCE_ROOT", "/root/reference")

_SOURCES = ["oracle_cs.cpp", "oracle_gen.cpp"]
_HEADERS = ["oracle_num.hpp", "oracle_ctx.hpp", "oracle_gen_prims.hpp", "upcg_oracle.h"]
_FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in _SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in _HEADERS]
    if force or _stale(ORACLE_SO, deps):
        cmd = ["g++", *_FLAGS, *srcs, "-o", ORACLE_SO + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    """Compile the reference's elementary cross sections; None if absent."""
    src = os.path.join(REFERENCE_ROOT, "src")
    inc = os.path.join(REFERENCE_ROOT, "include")
    units = [os.path.join(src, "UpcTwoPhotonDilep.cpp"), os.path.join(src, "UpcTwoPhotonALP.cpp")]
    if not all(os.path.exists(u) for u in units):
        return REF_SO if os.path.exists(REF_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.cpp")
    if force or _stale(REF_SO, units + [shim]):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
               "-I", inc, *units, shim, "-o", REF_SO + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(REF_SO + ".tmp", REF_SO)
    return REF_SO


REF_CS_SO = os.path.join(REF_DIR, "libupcref_cs.so")
_REF_CS_UNITS = ["UpcCrossSection.cpp", "UpcTwoPhotonDilep.cpp", "UpcTwoPhotonALP.cpp",
                 "UpcTwoPhotonDipion.cpp", "UpcTwoPhotonLbyL.cpp", "UpcPhotoNuclearVM.cpp"]


def build_ref_cs(force=False):
    """Compile the reference's UpcCrossSection against refshim/; None if the
    reference sources are absent (the prebuilt library is used if present)."""
    src = os.path.join(REFERENCE_ROOT, "src")
    inc = os.path.join(REFERENCE_ROOT, "include")
    units = [os.path.join(src, u) for u in _REF_CS_UNITS]
    if not all(os.path.exists(u) for u in units):
        return REF_CS_SO if os.path.exists(REF_CS_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    shim_dir = os.path.join(HERE, "refshim")
    shim = os.path.join(HERE, "ref_cs_shim.cpp")
    deps = units + [shim, os.path.join(HERE, "oracle_num.hpp")]
    deps += [os.path.join(shim_dir, f) for f in os.listdir(shim_dir) if f.endswith(".h")]
    if force or _stale(REF_CS_SO, deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-w", '-DCROSS_SEC_DIR="/nonexistent"', "-I", shim_dir, "-I", inc, *units, shim,
               "-lpthread", "-o", REF_CS_SO + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(REF_CS_SO + ".tmp", REF_CS_SO)
    return REF_CS_SO


REF_GEN_SO = os.path.join(REF_DIR, "libupcref_gen.so")


def build_ref_gen(force=False):
    """Compile the reference's event generator (src/UpcGenerator.cpp with the
    units of build_ref_cs) against refshim/ with ref_gen_shim.cpp (init and
    the event loop) and ref_out_shim.cpp (writeEvent's HepMC3 output) into
    oracle/_ref/libupcref_gen.so; None if the reference sources are absent.
    Pythia is off, as in a reference build without it."""
    src = os.path.join(REFERENCE_ROOT, "src")
    inc = os.path.join(REFERENCE_ROOT, "include")
    units = [os.path.join(src, u) for u in ["UpcGenerator.cpp"] + _REF_CS_UNITS]
    if not all(os.path.exists(u) for u in units):
        return REF_GEN_SO if os.path.exists(REF_GEN_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    shim_dir = os.path.join(HERE, "refshim")
    shim = os.path.join(HERE, "ref_gen_shim.cpp")
    out_shim = os.path.join(HERE, "ref_out_shim.cpp")
    deps = units + [shim, out_shim, os.path.join(HERE, "oracle_num.hpp"),
                    os.path.join(HERE, "oracle_gen_prims.hpp")]
    deps += [os.path.join(shim_dir, f) for f in os.listdir(shim_dir) if f.endswith(".h")]
    deps += [os.path.join(shim_dir, "gsl", f) for f in os.listdir(os.path.join(shim_dir, "gsl"))]
    if force or _stale(REF_GEN_SO, deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-w", '-DCROSS_SEC_DIR="/nonexistent"', "-I", shim_dir, "-I", inc, *units, shim,
               out_shim, "-lpthread", "-o", REF_GEN_SO + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(REF_GEN_SO + ".tmp", REF_GEN_SO)
    return REF_GEN_SO


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref_cs(force=True))
    print(build_ref_gen(force=True))
