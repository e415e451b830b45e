"""ctypes front end of the CPU restatement in oracle/hc_oracle.c.

TEST INFRASTRUCTURE ONLY. Imported by tests/, by __graft_entry__.smoke() (to
compare its results with), and by bench.py's CPU-baseline leg; never by the
product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
HIST_BINS = 1002
MAX_MODS = 15

ENTRY_DTYPE = np.dtype([("mass", "<f4"), ("seqid", "<u4"), ("sites", "<u8"),
                        ("modnum", "<u4"), ("pad", "<u4")])
RESULT_DTYPE = np.dtype([
    ("cpsms", "<u4"), ("idxoffset", "<i4"), ("psid", "<i4"), ("sharedions", "<u2"),
    ("totalions", "<u2"), ("hyperscore", "<f4"), ("mu", "<i4"), ("beta", "<i4"),
    ("minhyp", "<i4"), ("nexthyp", "<i4"), ("maxhyp", "<i4"), ("flags", "<u4"),
    ("reported", "<u4"), ("evalue", "<f8"), ("post_bytes", "<u8")])
assert ENTRY_DTYPE.itemsize == 24 and RESULT_DTYPE.itemsize == 64

FLAG_LGFACT_OOB, FLAG_HIST_OOB, FLAG_TAILFIT_OOB, FLAG_TAILFIT_EMPTY = 1, 2, 4, 8


class OrcParams(C.Structure):
    _fields_ = [("min_len", C.c_uint32), ("max_len", C.c_uint32), ("maxz", C.c_uint32),
                ("topmatches", C.c_uint32), ("scale", C.c_uint32), ("min_shp", C.c_uint32),
                ("min_cpsm", C.c_uint32), ("min_mass", C.c_uint32), ("max_mass", C.c_uint32),
                ("dF", C.c_uint32), ("base_int", C.c_int32), ("min_int", C.c_int32),
                ("dM", C.c_double), ("expect_max", C.c_double), ("nmods", C.c_uint32),
                ("vmods_per_pep", C.c_uint32), ("mod_mass", C.c_uint32 * MAX_MODS),
                ("mod_res", (C.c_char * 4) * MAX_MODS), ("mod_per_pep", C.c_uint32 * MAX_MODS),
                ("threads", C.c_uint32)]


class OrcLength(C.Structure):
    _fields_ = [("L", C.c_uint32), ("npep", C.c_uint32), ("n", C.c_uint32),
                ("seqs", C.c_void_p), ("entries", C.c_void_p), ("bA", C.c_void_p),
                ("iA", C.c_void_p)]


_lib = None


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    src = os.path.join(HERE, "hc_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        "-std=gnu11", src, "-o", LIB, "-lm"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.orc_make_entries.restype = C.c_int64
        _lib.orc_pep_mass.restype = C.c_float
        _lib.orc_mod_mass.restype = C.c_float
    return _lib


def to_cparams(p) -> OrcParams:
    c = OrcParams()
    for k in ("min_len", "max_len", "maxz", "topmatches", "scale", "min_shp", "min_cpsm",
              "min_mass", "max_mass", "dF", "base_int", "min_int", "vmods_per_pep", "threads"):
        setattr(c, k, int(getattr(p, k)))
    c.dM = float(p.dM)
    c.expect_max = float(p.expect_max)
    c.nmods = len(p.mods)
    for i, (res, _mass, per) in enumerate(p.mods):
        c.mod_mass[i] = p.mod_mass_scaled(i)
        c.mod_res[i].value = res.encode()[:4]
        c.mod_per_pep[i] = int(per)
    return c


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def make_entries(seqs: np.ndarray, L: int, p, sort: bool = True) -> np.ndarray:
    """Entries of one length (base peptides then variants), stably sorted by mass."""
    cp = to_cparams(p)
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    npep = seqs.shape[0]
    cap = max(16, npep * 4)
    while True:
        out = np.zeros(cap, dtype=ENTRY_DTYPE)
        n = lib().orc_make_entries(_ptr(seqs), C.c_uint32(npep), C.c_uint32(L), C.byref(cp),
                                   _ptr(out), C.c_int64(cap))
        if n >= 0:
            out = out[:n].copy()
            break
        cap *= 4
    if sort:
        lib().orc_sort_entries(_ptr(out), C.c_uint32(out.shape[0]))
    return out


def build_index(seqs: np.ndarray, L: int, entries: np.ndarray, p):
    cp = to_cparams(p)
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    entries = np.ascontiguousarray(entries, dtype=ENTRY_DTYPE)
    speclen = 2 * p.maxz * (L - 1)
    bA = np.zeros(p.max_mass * p.scale + 1, dtype=np.uint32)
    iA = np.zeros(entries.shape[0] * speclen, dtype=np.uint32)
    lib().orc_build_index(_ptr(seqs), C.c_uint32(L), _ptr(entries), C.c_uint32(entries.shape[0]),
                          C.byref(cp), _ptr(bA), _ptr(iA))
    return bA, iA


class OracleIndex:
    """All lengths of one database, as the oracle sees them."""

    def __init__(self, db: dict, p, entries: dict | None = None):
        self.p = p
        self.lengths = {}
        for L in range(p.min_len, p.max_len + 1):
            seqs = np.ascontiguousarray(db.get(L, np.zeros((0, L), np.uint8)), dtype=np.uint8)
            e = entries[L] if entries is not None else make_entries(seqs, L, p)
            e = np.ascontiguousarray(e, dtype=ENTRY_DTYPE)
            bA, iA = build_index(seqs, L, e, p)
            self.lengths[L] = dict(seqs=seqs, entries=e, bA=bA, iA=iA)

    def query(self, q, tie_rule: int = 1, threads: int | None = None, dM=None, want_hist=True):
        p = self.p
        cp = to_cparams(p)
        Ls = list(range(p.min_len, p.max_len + 1))
        arr = (OrcLength * len(Ls))()
        for i, L in enumerate(Ls):
            d = self.lengths[L]
            arr[i].L = L
            arr[i].npep = d["seqs"].shape[0]
            arr[i].n = d["entries"].shape[0]
            arr[i].seqs = d["seqs"].ctypes.data
            arr[i].entries = d["entries"].ctypes.data
            arr[i].bA = d["bA"].ctypes.data
            arr[i].iA = d["iA"].ctypes.data
        n = q.nspec
        out = np.zeros(n, dtype=RESULT_DTYPE)
        hist = np.zeros((n, HIST_BINS), dtype=np.uint32) if want_hist else None
        idx = np.ascontiguousarray(q.idx, dtype=np.uint32)
        moz = np.ascontiguousarray(q.moz, dtype=np.uint32)
        inten = np.ascontiguousarray(q.intensity, dtype=np.uint32)
        prec = np.ascontiguousarray(q.precurse, dtype=np.float32)
        if dM is None:
            dM = q.dM
        dMp = None if dM is None else np.ascontiguousarray(dM, dtype=np.float64)
        rc = lib().orc_query(arr, C.c_uint32(len(Ls)), C.byref(cp), _ptr(idx), _ptr(moz),
                             _ptr(inten), _ptr(prec), None if dMp is None else _ptr(dMp),
                             C.c_uint32(n), C.c_int(tie_rule), _ptr(out),
                             None if hist is None else _ptr(hist),
                             C.c_int(threads or p.threads))
        if rc != 0:
            raise RuntimeError(f"orc_query failed: {rc}")
        return out, hist
