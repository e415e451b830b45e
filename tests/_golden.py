"""Loader for the golden vectors recorded from the reference (tests/golden/*.npz)."""
import ast
import os
import zlib

import numpy as np

from hicops_gb300 import synthetic as S
from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("plain", "mods", "narrow", "plain20k")  # plain20k: the plain workload at its full size (20,000 peptides, 2,000 spectra)


def crc(a) -> int:
    return zlib.crc32(np.ascontiguousarray(a).tobytes()) & 0xFFFFFFFF


def load(name: str):
    z = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    kw = ast.literal_eval(str(z["params"][0]))
    p = S.SearchParams(threads=4, **kw)
    lens = [int(x) for x in z["lens"]]
    db, entries, crcs = {}, {}, {}
    off = eoff = 0
    for i, L in enumerate(lens):
        n = int(z["npep_per"][i])
        db[L] = z["seq_blob"][off:off + n * L].reshape(n, L).copy()
        off += n * L
        ne = int(z["nent"][i])
        e = np.zeros(ne, dtype=O.ENTRY_DTYPE)
        e["mass"] = z["ent_mass"][eoff:eoff + ne]
        e["seqid"] = z["ent_seqid"][eoff:eoff + ne]
        e["modnum"] = z["ent_modnum"][eoff:eoff + ne]
        e["sites"] = z["ent_sites"][eoff:eoff + ne]
        eoff += ne
        entries[L] = e
        crcs[L] = (int(z["index_crc"][i][0]), int(z["index_crc"][i][1]))
    nq = z["q_prec"].shape[0]
    q = S.QueryBatch(idx=z["q_idx"], moz=z["q_moz"], intensity=z["q_int"], precurse=z["q_prec"],
                     charges=np.full(nq, 2, np.int32), rtimes=np.zeros(nq, np.float32))
    rec = {k[4:]: z[k] for k in z.files if k.startswith("rec_")}
    return p, db, q, entries, crcs, rec


def hist_matches(hist: np.ndarray, rec: dict, rows: np.ndarray) -> bool:
    """The histograms of the reported spectra `rows` against the reference's: stored
    whole for the small cases, as one CRC per spectrum for the full-size one."""
    if "hist" in rec:
        return bool(np.array_equal(hist[rows], rec["hist"]))
    return bool(np.array_equal(np.array([crc(h) for h in hist[rows]], np.uint32), rec["hist_crc"]))
