"""MPSGCKP1 checkpoints of an MPS with its MPO (the format written by mpsg_dmrg_save and read by
mpsg_dmrg_load, little-endian):

    char[8] "MPSGCKP1"; u32 version (2; version-1 files have no settings record); u32 N
    version >= 2: u32 prec (mpsg_prec); u32 reorth; u32 lanmax; u64 updates (doStep calls made)
    per site s: u32 d; u64 charge[d]
                u32 Dl; u32 Dr; u32 nterms; nterms x {u32 wl, wr, out, in; f64 value}
                u32 nblocks; nblocks x {u64 q0, q1; u32 p; i32 rows, cols}; f64 data (blocks in key
                order, each column-major)
    u32 nlambda; nlambda x {i32 bond; u32 nblocks; nblocks x {u64 q; i32 n}; f64 data}
    char[8] "MPSGEND!"

Site tensors are dicts {(q0, q1, p): array}, lambdas {bond: {q: array}}, MPO tensors (terms, Dl, Dr)
with terms (wl, wr, out, in, value), charge maps lists of ints -- the structures of
mpstools_gb300.models and of the oracle.  This module is plain numpy (no GPU).
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC, END, VERSION = b"MPSGCKP1", b"MPSGEND!", 2
DEFAULT_SETTINGS = {"prec": 0, "reorth": 0, "lanmax": 500, "updates": 0}


def save(path, sites, mpo, itokeys, lambdas=None, settings=None):
    """settings: {"prec", "reorth", "lanmax", "updates"} of the run (default FP64, no
    reorthogonalisation, 500 Lanczos iterations, 0 updates)."""
    lambdas = lambdas or {}
    st = dict(DEFAULT_SETTINGS, **(settings or {}))
    with open(path, "wb") as f:
        f.write(MAGIC + struct.pack("<II", VERSION, len(sites)))
        f.write(struct.pack("<IIIQ", st["prec"], st["reorth"], st["lanmax"], st["updates"]))
        for s, site in enumerate(sites):
            ik = [int(q) for q in itokeys[s]]
            f.write(struct.pack("<I", len(ik)) + struct.pack(f"<{len(ik)}Q", *ik))
            terms, Dl, Dr = mpo[s]
            f.write(struct.pack("<III", Dl, Dr, len(terms)))
            for (wl, wr, out, inn, v) in sorted(terms, key=lambda t: (t[0], t[1], t[3], t[2])):
                f.write(struct.pack("<IIIId", wl, wr, out, inn, float(v)))
            keys = sorted(site)
            f.write(struct.pack("<I", len(keys)))
            for (q0, q1, p) in keys:
                r, c = np.shape(site[(q0, q1, p)])
                f.write(struct.pack("<QQIii", q0, q1, p, r, c))
            for k in keys:
                f.write(np.asarray(site[k], np.float64).reshape(-1, order="F").astype("<f8").tobytes())
        f.write(struct.pack("<I", len(lambdas)))
        for bond in sorted(lambdas):
            lam = lambdas[bond]
            qs = sorted(lam)
            f.write(struct.pack("<iI", bond, len(qs)))
            for q in qs:
                f.write(struct.pack("<Qi", q, len(lam[q])))
            for q in qs:
                f.write(np.asarray(lam[q], np.float64).astype("<f8").tobytes())
        f.write(END)


class _Reader:
    def __init__(self, data):
        self.b, self.o = data, 0

    def take(self, fmt):
        n = struct.calcsize(fmt)
        if self.o + n > len(self.b):
            raise ValueError("checkpoint file truncated")
        v = struct.unpack_from(fmt, self.b, self.o)
        self.o += n
        return v

    def array(self, n):
        v = self.take(f"<{n}d") if n else ()
        return np.array(v, np.float64)


def read_header(path):
    with open(path, "rb") as f:
        head = f.read(16)
    if head[:8] != MAGIC:
        raise ValueError("not an MPSG checkpoint file")
    version, N = struct.unpack("<II", head[8:16])
    return {"version": version, "N": N}


def read_settings(path):
    """The run settings of a version-2 file (the defaults for a version-1 file)."""
    with open(path, "rb") as f:
        head = f.read(36)
    if head[:8] != MAGIC:
        raise ValueError("not an MPSG checkpoint file")
    version, _ = struct.unpack("<II", head[8:16])
    if version < 2:
        return dict(DEFAULT_SETTINGS)
    p, r, lm, u = struct.unpack("<IIIQ", head[16:36])
    return {"prec": p, "reorth": r, "lanmax": lm, "updates": u}


def load(path):
    """Returns (sites, mpo, itokeys, lambdas)."""
    with open(path, "rb") as f:
        rd = _Reader(f.read())
    if bytes(rd.take("8s")[0]) != MAGIC:
        raise ValueError("not an MPSG checkpoint file")
    version, N = rd.take("<II")
    if version not in (1, 2):
        raise ValueError("unsupported checkpoint version")
    if version >= 2:
        rd.take("<IIIQ")
    sites, mpo, iks = [], [], []
    for _ in range(N):
        (d,) = rd.take("<I")
        iks.append(list(rd.take(f"<{d}Q")))
        Dl, Dr, nt = rd.take("<III")
        mpo.append(([tuple(rd.take("<IIIId")) for _ in range(nt)], Dl, Dr))
        (nb,) = rd.take("<I")
        heads = [rd.take("<QQIii") for _ in range(nb)]
        site = {}
        for (q0, q1, p, r, c) in heads:
            site[(q0, q1, p)] = rd.array(r * c).reshape((r, c), order="F")
        sites.append(site)
    lambdas = {}
    (nl,) = rd.take("<I")
    for _ in range(nl):
        bond, nb = rd.take("<iI")
        heads = [rd.take("<Qi") for _ in range(nb)]
        lambdas[bond] = {q: rd.array(n) for (q, n) in heads}
    if bytes(rd.take("8s")[0]) != END:
        raise ValueError("checkpoint end marker missing")
    return sites, mpo, iks, lambdas
