"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the unmodified reference DSLIM build + query (compiled from the
reference sources by oracle/ref/Makefile, driven by oracle/ref/ref_driver.cpp)
on small seeded synthetic cases and stores inputs and outputs as compressed
.npz files. Needs the reference sources (it builds oracle/_ref); the
fixtures it writes are what the tests read everywhere else.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hicops_gb300 import synthetic as S  # noqa: E402
from oracle import refrun  # noqa: E402

CASES = {
    # name: (params kwargs, peptides, spectra, db seed, query seed, query kwargs)
    "plain": (dict(maxz=2, dF=2, dM=100.0), 1500, 160, 0x60, 0x61, {}),
    "mods": (dict(maxz=3, dF=1, dM=500.0, vmods_per_pep=2, mods=[("M", 15.99, 2)]), 1500, 160, 0x70, 0x71, {}),
    "narrow": (dict(maxz=3, dF=1, dM=0.05, vmods_per_pep=2, mods=[("M", 15.99, 2)], min_cpsm=1),
               1500, 120, 0x80, 0x81, dict(peaks=(20, 150))),
}


def crc(a: np.ndarray) -> int:
    return zlib.crc32(np.ascontiguousarray(a).tobytes()) & 0xFFFFFFFF


# the plain workload at its full size (20,000 peptides, 2,000 spectra, dF 0.02 Da, dM 100 Da,
# fragment charges 1-2): the histograms are stored as one CRC per spectrum
FULL = {"plain20k": "plain-20k"}


def make(name: str) -> str:
    if name in FULL:
        p, npep, sdb, nq, sq, qkw = S.workload(FULL[name])
        p.threads = 4
        kw = {k: getattr(p, k) for k in ("maxz", "dF", "dM")}
    else:
        kw, npep, nq, sdb, sq, qkw = CASES[name]
        p = S.SearchParams(threads=4, **kw)
    db = S.make_database(npep, sdb, p)
    q = S.make_queries(db, nq, sq, p, **qkw)
    r = refrun.run(p, db, q, dump_index=True)
    lens = list(range(p.min_len, p.max_len + 1))
    seq_blob = np.concatenate([db[L].reshape(-1) for L in lens])
    npep_per = np.array([db[L].shape[0] for L in lens], np.uint32)
    ent = {k: np.concatenate([r["lengths"][L][k] for L in lens]) for k in ("mass", "seqid", "modnum", "sites")}
    nent = np.array([r["lengths"][L]["n"] for L in lens], np.uint32)
    crcs = np.array([[crc(r["lengths"][L]["bA"]), crc(r["lengths"][L]["iA"])] for L in lens], np.uint64)
    rec = r["records"]
    out = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(
        out,
        params=np.array([repr(kw)]), npep_total=np.array([npep]),
        lens=np.array(lens, np.uint32), seq_blob=seq_blob, npep_per=npep_per,
        q_idx=q.idx, q_moz=q.moz, q_int=q.intensity, q_prec=q.precurse,
        ent_mass=ent["mass"], ent_seqid=ent["seqid"], ent_modnum=ent["modnum"], ent_sites=ent["sites"],
        nent=nent, index_crc=crcs,
        **{f"rec_{f}": rec[f] for f in rec.dtype.names if not f.startswith("pad") and f != "hist"},
        **({"rec_hist_crc": np.array([crc(h) for h in rec["hist"][rec["reported"] == 1]], np.uint32)}
           if name in FULL else {"rec_hist": rec["hist"][rec["reported"] == 1]}))
    return out


if __name__ == "__main__":
    if not refrun.build():
        sys.exit("the reference sources are needed to regenerate the golden vectors")
    for n in list(CASES) + list(FULL):
        print(make(n), os.path.getsize(os.path.join(HERE, f"ref_{n}.npz")))
