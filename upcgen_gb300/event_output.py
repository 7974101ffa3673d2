"""Readers for the event files of ``UpcGenerator.writeEvents``.

* HepMC3 ASCII (format "hepmc"): the reference's ``events.hepmc``
  (WriterHepMC, include/UpcGenerator.h:192-242).
* Particle columns (format "columns"): the rows of the reference's ROOT tree
  ``particles`` (src/UpcGenerator.cpp:842-853) as a column file; the ROOT
  macro ``particles_to_root.C`` beside this file writes that tree from one.
  Layout: magic ``UPCGPRT1``; u32 version, u32 column count (9); u64 rows; per
  column {name[16], type 'I' (int32) or 'D' (float64), 7 pad bytes}; then the
  columns in that order, each padded to 8 bytes.
"""
import struct

import numpy as np

COLUMNS = ["eventNumber", "pdgCode", "particleID", "statusID", "motherID", "px", "py", "pz", "e"]


def read_particle_columns(path):
    """{column name: numpy array} of a column file."""
    raw = open(path, "rb").read()
    if raw[:8] != b"UPCGPRT1":
        raise ValueError("not a particle column file")
    version, ncol = struct.unpack_from("=2I", raw, 8)
    (nrows,) = struct.unpack_from("=Q", raw, 16)
    if version != 1:
        raise ValueError(f"version {version}")
    off = 24 + 24 * ncol
    out = {}
    for c in range(ncol):
        d = raw[24 + 24 * c:48 + 24 * c]
        name = d[:16].rstrip(b"\0").decode()
        dt = {b"I": np.int32, b"D": np.float64}[d[16:17]]
        size = np.dtype(dt).itemsize * nrows
        out[name] = np.frombuffer(raw, dtype=dt, count=nrows, offset=off).copy()
        off += (size + 7) // 8 * 8
    if off != len(raw):
        raise ValueError(f"file has {len(raw)} bytes, layout {off}")
    return out


def read_hepmc3(path_or_text):
    """Events of a HepMC3 ASCII listing as the reference writes it:
    ([(event, vertices, particles)], particle rows [[id, mother, pdg, px, py,
    pz, e, m, status], ...] as float64)."""
    text = path_or_text
    if "\n" not in text:
        text = open(text).read()
    events, rows = [], []
    for line in text.split("\n"):
        if line.startswith("E "):
            _, a, b, c = line.split()
            events.append((int(a), int(b), int(c)))
        elif line.startswith("P "):
            rows.append([float(x) for x in line.split()[1:]])
    return events, np.array(rows, dtype=np.float64).reshape(-1, 9)
