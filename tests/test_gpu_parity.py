"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bit-exact: entries and their order, bA, iA, cpsms, histograms, top hit
(length, psid, shared ions), hyperscore. Tail-fit ints mu/beta exact for
>= 99 % of reported spectra and |delta log10 e| <= 0.05 for all (the device
log10/pow may differ from the host's in the last bit).
"""
import numpy as np
import pytest

from tests._util import case, compare
from hicops_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dslim():
    from hicops_gb300 import dslim as D
    return D


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle as O
    return O


@pytest.mark.parametrize("name,npep,nq,seed", [("plain", 3000, 300, 101), ("mods", 3000, 300, 202)])
def test_index_bitexact(dslim, orc, name, npep, nq, seed):
    p, db, q = case(name, npep, nq, seed)
    ix = dslim.Index(p)
    ix.construct_all(db)
    for L in range(p.min_len, p.max_len + 1):
        e, bA, iA = ix.export(L)
        oe = orc.make_entries(db[L], L, p)          # stable by mass, generation order
        assert e.shape == oe.shape
        assert np.array_equal(e.view(np.uint8), oe.view(np.uint8)), f"entries differ at L={L}"
        obA, oiA = orc.build_index(db[L], L, oe, p)
        assert np.array_equal(bA, obA), f"bA differs at L={L}"
        assert np.array_equal(iA, oiA), f"iA differs at L={L}"
    ix.close()


@pytest.mark.parametrize("mods,vmods", [([("M", 15.99, 2), ("STY", 79.97, 1)], 3),
                                         ([("M", 15.99, 1), ("NQ", 0.98, 2), ("STY", 79.97, 3)], 4),
                                         ([("M", 15.99, 3)], 1),
                                         ([("M", 15.99, 2), S.NTERM_ACETYL], 3)])
def test_device_enumeration_multi_mod(dslim, orc, mods, vmods):
    """Entries enumerated on the device (several mod conditions, per-condition
    limits, a total limit) equal the host enumeration, sorted stably by mass."""
    p = S.SearchParams(maxz=2, dF=1, dM=100.0, vmods_per_pep=vmods, mods=mods)
    db = S.make_database(4000, 77 + vmods, p)
    ix = dslim.Index(p)
    ix.construct_all(db)
    nvar = 0
    for L in range(p.min_len, p.max_len + 1):
        e = ix.entries(L)
        oe = orc.make_entries(db[L], L, p)
        assert np.array_equal(e.view(np.uint8), oe.view(np.uint8)), f"entries differ at L={L}"
        nvar += int((oe["modnum"] != 0).sum())
    assert nvar > 1000
    ix.close()


@pytest.mark.parametrize("name,npep,nq,seed", [("plain", 3000, 400, 303), ("mods", 3000, 400, 404)])
def test_query_parity(dslim, orc, name, npep, nq, seed):
    p, db, q = case(name, npep, nq, seed)
    ix = dslim.Index(p)
    ix.construct_all(db)
    res, hist = ix.query(q)
    oi = orc.OracleIndex(db, p)
    ores, ohist = oi.query(q, tie_rule=1)
    st = compare(res, hist, ores, ohist)
    assert st["reported"] > 0
    ix.close()


def test_query_parity_nterm_acetyl(dslim, orc):
    """The N-terminal acetylation extension (variants, b-ion shift, precursor mass)
    on the device equals the oracle's restatement of the same rules, and spectra
    made from acetylated peptides find acetylated entries."""
    p = S.SearchParams(maxz=3, dF=1, dM=100.0, threads=8, vmods_per_pep=3, mods=[("M", 15.99, 2), S.NTERM_ACETYL])
    db = S.make_database(3000, 606, p)
    q = S.make_queries(db, 400, 607, p)
    ix = dslim.Index(p)
    ix.construct_all(db)
    for L in (p.min_len, 20, p.max_len):
        e = ix.entries(L)
        oe = orc.make_entries(db[L], L, p)
        assert np.array_equal(e.view(np.uint8), oe.view(np.uint8)), f"entries differ at L={L}"
    res, hist = ix.query(q)
    oi = orc.OracleIndex(db, p)
    ores, ohist = oi.query(q, tie_rule=1)
    compare(res, hist, ores, ohist)
    sid, mod, site = ix.identity(res)
    acetyl = (site >> np.uint64(63)) & np.uint64(1) == 1
    assert acetyl.sum() >= 20, int(acetyl.sum())
    ix.close()


def test_query_parity_loaded_index(dslim, orc):
    """Query over a host-built index loaded as-is (hc_dslim_load)."""
    p, db, q = case("mods", 2000, 200, 505)
    oi = orc.OracleIndex(db, p)
    ix = dslim.Index(p)
    for L, d in oi.lengths.items():
        ix.load(L, d["seqs"], d["entries"], d["bA"], d["iA"])
    res, hist = ix.query(q)
    ores, ohist = oi.query(q, tie_rule=1)
    compare(res, hist, ores, ohist)
    ix.close()


def test_query_parity_mixed_windows(dslim, orc):
    """Per-spectrum precursor tolerances (10 ppm / 50 Da / 500 Da)."""
    p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
    db = S.make_database(3000, 606, p)
    q = S.make_queries(db, 400, 607, p, peaks=(20, 150),
                       window_mix=[(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)])
    ix = dslim.Index(p)
    ix.construct_all(db)
    res, hist = ix.query(q)
    ores, ohist = orc.OracleIndex(db, p).query(q, tie_rule=1)
    compare(res, hist, ores, ohist)
    ix.close()


def test_wide_path(dslim, orc):
    """Intensities >= 2^17 cannot use the packed scorecard: the wide kernel must agree."""
    p, db, q = case("plain", 2000, 200, 707, base_int=1000000, min_int=10000)
    q2 = S.make_queries(db, 200, 708, p)
    ix = dslim.Index(p)
    ix.construct_all(db)
    res, hist = ix.query(q2)
    assert (res["flags"] & 0x100).any(), "wide path not exercised"
    ores, ohist = orc.OracleIndex(db, p).query(q2, tie_rule=1)
    compare(res, hist, ores, ohist)
    ix.close()


def test_count_overflow_goes_wide(dslim, orc):
    """Peaks that share buckets can push a candidate's ion count past 127. Such
    spectra keep the atomics that return the old scorecard words, see the
    overflow and are redone wide; spectra with every peak in its own buckets
    use the other form. Both must agree with the oracle."""
    p = S.SearchParams(maxz=3, dF=1, dM=500.0)
    db = S.make_database(2000, 919, p)
    poly = np.frombuffer(("G" * 39 + "K").encode(), np.uint8).reshape(1, 40)
    db[40] = np.concatenate([poly, db[40]]) if db[40].shape[0] else poly.copy()
    ix = dslim.Index(p)
    ix.construct_all(db)
    e, bA, iA = ix.export(40)
    k = int(np.nonzero(e["seqid"] == 0)[0][0])      # the poly-G entry
    speclen = 2 * p.maxz * 39
    ids = np.nonzero(iA // speclen == k)[0]
    ions = iA[ids] % speclen
    bkt = np.searchsorted(bA, ids, side="right") - 1  # bucket of each of its postings
    bkeys, nb_ions = np.unique(bkt[ions < speclen // 2], return_counts=True)
    top = bkeys[np.argsort(-nb_ions, kind="stable")[:33]]
    assert 3 * int(np.sort(nb_ions)[::-1][:33].sum()) >= 128   # the b count the first spectrum reaches
    thrice = np.repeat(top, 3)                          # every key three times: lists share buckets
    once = bkeys[np.arange(0, bkeys.size, 3)][:100]     # spread keys: buckets of their own
    spectra = [thrice, once]
    idx = np.cumsum([0] + [s.size for s in spectra]).astype(np.uint32)
    moz = np.concatenate(spectra).astype(np.uint32)
    inten = np.concatenate([np.linspace(1000, 100000, s.size).astype(np.uint32) for s in spectra])
    prec = np.full(len(spectra), float(e["mass"][k]), np.float32)
    q = S.QueryBatch(idx=idx, moz=moz, intensity=inten, precurse=prec,
                     charges=np.full(len(spectra), 2, np.int32), rtimes=np.zeros(len(spectra), np.float32))
    res, hist = ix.query(q)
    assert res["flags"][0] & 0x100, "count overflow not detected"
    assert not res["flags"][1] & 0x100
    ores, ohist = orc.OracleIndex(db, p).query(q, tie_rule=1)
    compare(res, hist, ores, ohist)
    ix.close()


def test_small_tiles(dslim, orc):
    """Many scorecard tiles per length (the smallest tile, windows several tiles wide)."""
    p, db, q = case("mods", 200000, 100, 808)
    ix = dslim.Index(p)
    ix.construct_all(db)
    ix.set_tuning(tile=2048, threads=256)
    res, hist = ix.query(q)
    ores, ohist = orc.OracleIndex(db, p).query(q, tie_rule=1)
    compare(res, hist, ores, ohist)
    ix.close()


@pytest.mark.parametrize("threads,ppw", [(64, 1), (128, 2)])
def test_small_blocks(dslim, orc, threads, ppw):
    """Blocks smaller than a third of the (peak, bin) lists: list bounds past
    the per-thread prefetch slots are computed directly. The batch also has
    candidates in histogram bins from 256 on (hyperscores of 25.6 and more),
    which the kernel adds to the output histogram directly."""
    p, db, q = case("mods", 20000, 120, 818)
    ix = dslim.Index(p)
    ix.construct_all(db)
    ix.set_tuning(tile=4096, threads=threads, pairs_per_warp=ppw, ctas_per_sm=1)
    res, hist = ix.query(q)
    ores, ohist = orc.OracleIndex(db, p).query(q, tie_rule=1)
    assert (ohist.reshape(q.nspec, -1)[:, 256:] > 0).any()
    compare(res, hist, ores, ohist)
    ix.close()


@pytest.mark.parametrize("cap", [0, 1, 128])
def test_undecided_queue_capacity(dslim, orc, cap):
    """Candidates whose sign or histogram bin the float estimate leaves open:
    evaluated in place (cap 0), mostly in place once a one-entry queue is full,
    or queued and resolved at the spectrum's end; all give the oracle's results."""
    p, db, q = case("mods", 20000, 150, 828)
    ix = dslim.Index(p)
    ix.construct_all(db)
    ix.set_tuning(defer_cap=cap)
    res, hist = ix.query(q)
    ores, ohist = orc.OracleIndex(db, p).query(q, tie_rule=1)
    compare(res, hist, ores, ohist)
    ix.close()


def test_empty_and_edge_batches(dslim, orc):
    p, db, q = case("plain", 1000, 50, 909)
    ix = dslim.Index(p)
    ix.construct_all(db)
    # empty batch
    e = q.slice(0, 0)
    r0, _ = ix.query(e)
    assert r0.shape == (0,)
    # spectra with no peaks, with a single peak, with peaks at the bin limits
    nz = S.QueryBatch(idx=np.array([0, 0, 1, 4], np.uint32),
                      moz=np.array([50000, 0, 2, 499998], np.uint32),
                      intensity=np.array([100000, 5, 5, 5], np.uint32),
                      precurse=np.array([1500.0, 1200.0, 2000.0], np.float32),
                      charges=np.array([2, 2, 2], np.int32), rtimes=np.zeros(3, np.float32))
    r, h = ix.query(nz)
    orr, oh = orc.OracleIndex(db, p).query(nz, tie_rule=1)
    compare(r, h, orr, oh)
    ix.close()
