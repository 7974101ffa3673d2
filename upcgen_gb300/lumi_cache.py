"""Reader for the luminosity cache files written by ``upcg_init`` when the
cache is on (``UpcGenerator.setLumiCache(True)``).

The file replaces the reference's ``twoPhotonLumi.root`` /
``twoPhotonLumiPol.root`` (src/UpcCrossSection.cpp:463-592): the same table
(L dm dy on the left-edge grid, ``hD2LDMDY`` bin (im+1, iy+1) = table[im][iy];
polarized: ``hD2LDMDY_s`` and ``hD2LDMDY_p``), keyed by every input of the
table.  ``lumi_cache_to_root.C`` beside this file turns one into that ROOT file
for tools that read it.

Layout (host byte order, fields 8-byte aligned): magic ``UPCGLUM1``; u32
version, ntab, nm, ny; u64 key length, key text zero-padded to 8 bytes; u64
FNV-1a 64 of the payload; f64 payload [ntab][nm][ny].
"""
import re
import struct

import numpy as np

MAGIC = b"UPCGLUM1"
VERSION = 1


def fnv1a64(data):
    """FNV-1a 64 (offset basis 0xcbf29ce484222325, prime 0x100000001b3)."""
    h = 0xcbf29ce484222325
    for b in bytes(data):
        h ^= b
        h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


_RANGE = re.compile(r"; (m|y) \[([^,\]]+), ([^\]]+)\] bins (\d+)")


def parse_key(key):
    """Axis ranges of the table from the key text: {"m": (lo, hi, n), "y": ...}."""
    out = {}
    for ax, lo, hi, n in _RANGE.findall(key):
        out[ax] = (float.fromhex(lo), float.fromhex(hi), int(n))
    return out


def read_lumi_cache(path, verify=True):
    """Returns {"key": str, "tables": float64 [ntab][nm][ny], "m": (lo, hi, nm),
    "y": (lo, hi, ny)}; raises ValueError on a malformed or corrupted file.
    verify=False skips the payload checksum (pure Python: about 0.2 s per MB)."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:8] != MAGIC:
        raise ValueError("not a luminosity cache file")
    version, ntab, nm, ny = struct.unpack_from("=4I", raw, 8)
    if version != VERSION:
        raise ValueError(f"cache version {version}, reader {VERSION}")
    (klen,) = struct.unpack_from("=Q", raw, 24)
    kpad = (klen + 7) // 8 * 8
    key = raw[32:32 + klen].decode()
    off = 32 + kpad
    (csum,) = struct.unpack_from("=Q", raw, off)
    off += 8
    n = ntab * nm * ny
    payload = raw[off:]
    if len(payload) != 8 * n:
        raise ValueError(f"payload has {len(payload)} bytes, expected {8 * n}")
    if verify and fnv1a64(payload) != csum:
        raise ValueError("payload checksum mismatch")
    tables = np.frombuffer(payload, dtype=np.float64).reshape(ntab, nm, ny).copy()
    axes = parse_key(key)
    return {"key": key, "tables": tables, "m": axes.get("m"), "y": axes.get("y")}
