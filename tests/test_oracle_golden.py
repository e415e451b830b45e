"""The CPU oracle against the golden vectors recorded from the reference.

Pins the restatement: with the reference's own entry order, bA/iA match the
reference byte for byte (CRC), and every reported spectrum's top hit (heap
tie rule), shared ions, cpsms, hyperscore, histogram, tail-fit ints and
e-value equal the reference's exactly.
"""
import numpy as np
import pytest

from tests._golden import CASES, crc, hist_matches, load
from oracle import oracle as O


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    p, db, q, entries, crcs, rec = load(name)
    oi = O.OracleIndex(db, p, entries=entries)
    for L, (cb, ci) in crcs.items():
        assert crc(oi.lengths[L]["bA"]) == cb, f"bA crc differs at L={L}"
        assert crc(oi.lengths[L]["iA"]) == ci, f"iA crc differs at L={L}"
    res, hist = oi.query(q, tie_rule=0)
    rep = rec["reported"] == 1
    assert np.array_equal(res["reported"] == 1, rep)
    assert rep.sum() > 10
    i = np.nonzero(rep)[0]
    for a, b in [("npsms", "cpsms"), ("psid", "psid"), ("idxoffset", "idxoffset"),
                 ("sharedions", "sharedions"), ("totalions", "totalions"), ("mu", "mu"), ("beta", "beta"),
                 ("minhyp", "minhyp"), ("nexthyp", "nexthyp"), ("maxhyp", "maxhyp")]:
        assert np.array_equal(rec[a][i], res[b][i]), a
    assert np.array_equal(rec["hyperscore"][i], res["hyperscore"][i])
    assert np.array_equal(rec["e_x"][i], res["evalue"][i])
    assert hist_matches(hist, rec, i)


@pytest.mark.parametrize("name", CASES)
def test_oracle_entries_match_reference_set(name):
    """Variant enumeration: same entries (as a multiset) as the reference produced."""
    p, db, q, entries, crcs, rec = load(name)
    for L, e in entries.items():
        mine = O.make_entries(db[L], L, p)
        key = lambda x: np.sort(x["mass"].view(np.uint32).astype(np.uint64) << 32 | x["seqid"].astype(np.uint64)
                                ^ (x["sites"] * np.uint64(2654435761)) ^ x["modnum"].astype(np.uint64))
        assert mine.shape == e.shape
        assert np.array_equal(key(mine), key(e)), L
