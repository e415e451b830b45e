"""Shared helpers for the parity tests (comparison against the oracle)."""
import numpy as np

from hicops_gb300 import synthetic as S
from hicops_gb300 import _lib as HL

CMP_INT = ("cpsms", "idxoffset", "psid", "sharedions", "totalions", "minhyp", "nexthyp", "maxhyp",
           "reported", "post_bytes")


def case(name: str, npep: int, nq: int, seed: int, **kw):
    if name == "plain":
        p = S.SearchParams(maxz=2, dF=2, dM=100.0, threads=8)
    elif name == "mods":
        p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
    else:
        raise KeyError(name)
    for k, v in kw.items():
        setattr(p, k, v)
    db = S.make_database(npep, seed, p)
    q = S.make_queries(db, nq, seed + 1, p)
    return p, db, q


def compare(gpu: np.ndarray, ghist: np.ndarray, orc: np.ndarray, ohist: np.ndarray,
            fit_exact_min: float = 0.99) -> dict:
    """Assert the parity rules; returns statistics."""
    assert gpu.shape == orc.shape
    stats = {"n": int(gpu.shape[0])}
    for f in CMP_INT:
        bad = np.nonzero(gpu[f] != orc[f])[0]
        assert bad.size == 0, f"{f} differs at {bad[:10]}: gpu {gpu[f][bad[:5]]} oracle {orc[f][bad[:5]]}"
    assert np.array_equal(gpu["hyperscore"], orc["hyperscore"]), "hyperscore differs"
    assert np.array_equal(ghist, ohist), "histograms differ"
    fl_mask = ~np.uint32(HL.FLAG_WIDE)
    assert np.array_equal(gpu["flags"] & fl_mask, orc["flags"]), "flags differ"
    rep = orc["reported"] == 1
    same_fit = (gpu["mu"] == orc["mu"]) & (gpu["beta"] == orc["beta"])
    stats["fit_exact"] = float(same_fit[rep].mean()) if rep.any() else 1.0
    assert stats["fit_exact"] >= fit_exact_min, stats
    ok = rep & (orc["evalue"] > 0) & (gpu["evalue"] > 0)
    d = np.abs(np.log10(gpu["evalue"][ok]) - np.log10(orc["evalue"][ok]))
    stats["dlog10e_max"] = float(d.max()) if d.size else 0.0
    assert stats["dlog10e_max"] <= 0.05, stats
    stats["reported"] = int(rep.sum())
    return stats
