"""The oracle against the compiled reference on fresh seeded workloads.

Runs only where the reference was built (oracle/_ref, made by build() where
the reference sources are mounted); the golden-vector tests cover the same
ground everywhere else.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import refrun
from hicops_gb300 import synthetic as S

pytestmark = pytest.mark.skipif(not refrun.available(), reason="reference oracle not built here")


def _ents(r, p):
    out = {}
    for L in range(p.min_len, p.max_len + 1):
        d = r["lengths"][L]
        e = np.zeros(d["n"], dtype=O.ENTRY_DTYPE)
        for k in ("mass", "seqid", "modnum", "sites"):
            e[k] = d[k]
        out[L] = e
    return out


@pytest.mark.parametrize("wl,nq", [("plain-20k", 2000)])
def test_full_plain_workload(wl, nq):
    p, npep, sdb, _, sq, kw = S.workload(wl)
    p.threads = 8
    db = S.make_database(npep, sdb, p)
    q = S.make_queries(db, nq, sq, p, **kw)
    r = refrun.run(p, db, q, dump_index=True)
    oi = O.OracleIndex(db, p, entries=_ents(r, p))
    for L in oi.lengths:
        assert np.array_equal(oi.lengths[L]["bA"], r["lengths"][L]["bA"])
        assert np.array_equal(oi.lengths[L]["iA"], r["lengths"][L]["iA"])
    res, hist = oi.query(q, tie_rule=0)
    rec = r["records"]
    rep = rec["reported"] == 1
    assert np.array_equal(rep, res["reported"] == 1)
    i = np.nonzero(rep)[0]
    for a, b in [("npsms", "cpsms"), ("psid", "psid"), ("idxoffset", "idxoffset"), ("sharedions", "sharedions"),
                 ("mu", "mu"), ("beta", "beta"), ("maxhyp", "maxhyp"), ("hyperscore", "hyperscore"),
                 ("e_x", "evalue")]:
        assert np.array_equal(rec[a][i], res[b][i]), a
    assert np.array_equal(rec["hist"][i], hist[i])


def test_mods_open_search():
    p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
    db = S.make_database(6000, 77, p)
    q = S.make_queries(db, 600, 78, p)
    r = refrun.run(p, db, q, dump_index=True)
    oi = O.OracleIndex(db, p, entries=_ents(r, p))
    res, hist = oi.query(q, tie_rule=0)
    rec = r["records"]
    i = np.nonzero(rec["reported"] == 1)[0]
    assert np.array_equal(rec["reported"] == 1, res["reported"] == 1)
    for a, b in [("npsms", "cpsms"), ("psid", "psid"), ("mu", "mu"), ("beta", "beta"), ("e_x", "evalue")]:
        assert np.array_equal(rec[a][i], res[b][i]), a
    assert np.array_equal(rec["hist"][i], hist[i])
