"""GPU tests of MS2 ingestion with device peak picking (hc_ms2_open /
hc_ms2_extract, the reference's MSQuery::initialize / extractbatch /
readspectrum / pickpeaks, msquery.cpp:88-569): bit-exact against the
reference's outputs (golden vectors) and against the restatement in
oracle/ms2.py on fresh seeded files, in whole and in chunks; the reader's
error codes; and MS2 text -> device batch -> search -> PSM TSV end to end."""
import os

import numpy as np
import pytest

from oracle import ms2 as M
from tests import _ms2cases as MC
from tests._util import case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS = ("idx", "moz", "intensity", "precurse", "charges", "rtimes")


def _index(scale=100, base_int=100000, min_int=1000):
    from hicops_gb300 import dslim
    from hicops_gb300 import synthetic as S
    p = S.SearchParams(maxz=2, dF=2, dM=100.0)
    p.scale, p.base_int, p.min_int = scale, base_int, min_int
    return dslim.Index(p)


def _device_batch(ix, path, chunk=None):
    from hicops_gb300 import dslim
    r = dslim.MSQuery(ix).initialize(path)
    n = r.getQAcount()
    parts = []
    if chunk is None:
        b, rem = r.extractbatch(max(n, 1))
        assert rem == 0
        parts.append(b)
    else:
        rem = n
        while rem > 0:
            b, rem = r.extractbatch(chunk)
            parts.append(b)
    r.DeinitQueryFile()
    idx = [np.zeros(1, np.uint32)]
    base = 0
    for b in parts:
        idx.append(b.idx[1:] + base)
        base += int(b.idx[-1])
    return dict(idx=np.concatenate(idx).astype(np.uint32),
                moz=np.concatenate([b.moz for b in parts]).astype(np.uint32),
                intensity=np.concatenate([b.intensity for b in parts]).astype(np.uint32),
                precurse=np.concatenate([b.precurse for b in parts]).astype(np.float32),
                charges=np.concatenate([b.charges for b in parts]).astype(np.int32),
                rtimes=np.concatenate([b.rtimes for b in parts]).astype(np.float32))


def _same(a: dict, b: dict):
    for k in KEYS:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.dtype.itemsize == y.dtype.itemsize and np.array_equal(x.view(np.uint8), y.view(np.uint8)), k


@pytest.mark.parametrize("name", ["edge", "lf-default", "crlf-coarse"])
@pytest.mark.parametrize("chunk", [None, 7])
def test_matches_reference_golden(name, chunk, tmp_path):
    g = np.load(os.path.join(GOLDEN, f"ms2_{name}.npz"))
    path = tmp_path / "g.ms2"
    path.write_bytes(g["ms2"].tobytes())
    ix = _index(*[int(v) for v in g["pick"]])
    _same(_device_batch(ix, str(path), chunk), g)
    ix.close()


@pytest.mark.parametrize("name,seed,chunk", [("lf-default", 21, None), ("crlf-fine", 22, 64),
                                             ("lf-coarse", 23, 1000)])
def test_matches_oracle_random(name, seed, chunk, tmp_path):
    path = str(tmp_path / "r.ms2")
    pick = MC.write_case(path, name, seed, nspec=400, max_peaks=600)
    st, o = M.read_ms2(path, *pick)
    assert st == 0
    ix = _index(*pick)
    _same(_device_batch(ix, path, chunk), o)
    ix.close()


def test_long_spectra(tmp_path):
    """Spectra of several thousand raw peaks with few distinct intensities."""
    path = str(tmp_path / "long.ms2")
    rng = np.random.default_rng(7)
    specs = []
    for s in range(12):
        npk = int(rng.integers(2000, 6000))
        lv = np.round(rng.uniform(1, 900, 40), 2)
        specs.append((s + 1, "1500.5", 2, "3.0", [(f"{a:.4f}", f"{b:.2f}") for a, b in
                                                   zip(rng.uniform(100, 2000, npk), rng.choice(lv, npk))]))
    M.write_ms2(path, specs)
    st, o = M.read_ms2(path, 100, 100000, 1000)
    ix = _index()
    _same(_device_batch(ix, path), o)
    ix.close()


def test_errors(tmp_path):
    from hicops_gb300 import dslim
    from hicops_gb300._lib import HcError
    ix = _index()
    with pytest.raises(HcError) as e:
        dslim.MSQuery(ix).initialize(str(tmp_path / "missing.ms2"))
    assert e.value.status == -3013
    p = tmp_path / "nopeaks.ms2"
    p.write_text("H\tx\nS\t1\t1\t500\nZ\t2\t999\n")
    with pytest.raises(HcError) as e:
        dslim.MSQuery(ix).initialize(str(p))
    assert e.value.status == -3004
    # no 'S' line: no spectra, as the reference counts them
    p2 = tmp_path / "noscan.ms2"
    p2.write_text("100.0 5.0\n")
    r = dslim.MSQuery(ix).initialize(str(p2))
    assert r.getQAcount() == 0
    b, rem = r.extractbatch(10)
    assert b.nspec == 0 and rem == 0
    r.DeinitQueryFile()
    ix.close()


def test_ms2_to_psms_end_to_end(tmp_path):
    """Queries written as MS2 text, read and picked on the device, searched and
    printed give the results of searching the batch directly."""
    from hicops_gb300 import dslim
    p, db, q = case("mods", 5000, 300, 913)
    ix = dslim.Index(p)
    ix.construct_all(db)
    path = str(tmp_path / "q.ms2")
    MC.write_queries(path, q, p.scale)
    r = dslim.MSQuery(ix).initialize(path)
    assert r.getQAcount() == q.nspec
    outs, n_rep = [], 0
    tsv = str(tmp_path / "psms.tsv")
    rem, base = q.nspec, 0
    while rem > 0:
        b, rem = r.extractbatch(128)
        res, _ = ix.query(b, want_hist=False)
        ix.write_psms(tsv, res, b, file_label="q.ms2", spec_base=base, append=base > 0)
        outs.append(res)
        base += b.nspec
        n_rep += int((res["reported"] == 1).sum())
    r.DeinitQueryFile()
    got = np.concatenate(outs)
    ref, _ = ix.query(q, want_hist=False)
    for f in ("reported", "psid", "idxoffset", "sharedions", "totalions", "hyperscore", "cpsms"):
        assert np.array_equal(got[f], ref[f]), f
    assert np.array_equal(got["evalue"][ref["reported"] == 1], ref["evalue"][ref["reported"] == 1])
    lines = open(tsv).read().splitlines()
    assert len(lines) == 1 + n_rep and n_rep > 0
    scans = [int(l.split("\t")[1]) for l in lines[1:]]
    assert scans == [int(i) + 1 for i in np.nonzero(ref["reported"] == 1)[0]]
    ix.close()
